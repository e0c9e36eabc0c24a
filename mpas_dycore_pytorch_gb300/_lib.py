"""ctypes binding of the C ABI in ``include/mpasg.h`` (``libmpasg.so``).

The struct layouts below mirror the header field by field.  The library is loaded from
the package directory (built in tree by ``build.py``); there is no fallback: when the
library is missing the import of the device path raises ``MpasExtensionMissingError``.
"""

from __future__ import annotations

import ctypes as C
import pathlib

from .errors import MpasConfigError, MpasDeviceError, MpasExtensionMissingError, MpasNumericalError

LIB_PATH = pathlib.Path(__file__).resolve().parent / "libmpasg.so"
ABI_VERSION = 4

MESH_INT_DIMS = ("nCells", "nEdges", "nVertices", "nVertLevels", "maxEdges", "maxEdges2",
                 "vertexDegree", "nAdvMax", "flatTerrain", "reserved0")
MESH_DOUBLES = ("cf1", "cf2", "cf3")
MESH_INT_PTRS = ("nEdgesOnCell", "edgesOnCell", "cellsOnCell", "verticesOnCell", "kiteForCell",
                 "cellsOnEdge", "verticesOnEdge", "nEdgesOnEdge", "edgesOnEdge",
                 "nAdvCellsForEdge", "advCellsForEdge", "edgesOnVertex")
MESH_DBL_PTRS = ("edgesOnCell_sign", "edgesOnVertex_sign", "dcEdge", "dvEdge", "invDcEdge",
                 "invDvEdge", "invAreaCell", "invAreaTriangle", "kiteAreasOnVertex",
                 "weightsOnEdge", "adv_coefs", "adv_coefs_3rd", "adv_coefs_p", "adv_coefs_m",
                 "defc_a", "defc_b", "fEdge",
                 "fVertex", "meshScalingDel2", "meshScalingDel4", "latCell", "lonCell",
                 "coeffs_reconstruct", "zb_cell", "zb3_cell", "zxu", "zz", "dss", "rho_base",
                 "theta_base", "rdzw", "rdzu", "fzm", "fzp", "fnm", "fnp", "rdnw",
                 "ref_theta", "ref_theta_w4", "ref_theta_w3", "ref_theta_w2")

CONFIG_DOUBLES = ("dt", "epssm", "smdiv", "len_disp", "coef_3rd_order", "c_s", "visc4_2dsmag",
                  "del4u_div_factor", "apvm_upwinding", "h_mom_eddy_visc4", "h_theta_eddy_visc4")
CONFIG_INTS = ("time_integration_order", "number_of_sub_steps", "dynamics_split_steps",
               "monotonic", "horiz_mixing_smagorinsky", "num_scalars", "moist_start", "moist_end",
               "precision", "tile_tend_u")
PRECISIONS = {"float64": 0, "mixed": 1}

# (name, kind) in header order; kind names the row space: e/c/cw/v/cs/es/cws/L/cL/cLw/...
FIELDS = (
    ("u", "e"), ("v", "e"), ("ru", "e"), ("ruAvg", "e"), ("h_edge", "e"), ("pv_edge", "e"),
    ("w", "cw"), ("rw", "cw"), ("wwAvg", "cw"),
    ("theta_m", "c"), ("rho_zz", "c"), ("rho_p", "c"), ("rtheta_p", "c"), ("rtheta_base", "c"),
    ("exner", "c"), ("exner_base", "c"), ("pressure_p", "c"), ("pressure_base", "c"),
    ("divergence", "c"), ("ke", "c"), ("rt_diabatic_tend", "c"),
    ("uReconstructX", "c"), ("uReconstructY", "c"), ("uReconstructZ", "c"),
    ("uReconstructZonal", "c"), ("uReconstructMeridional", "c"),
    ("vorticity", "v"),
    ("scalars", "cs"),
    ("ru_save", "e"), ("ruAvg_split", "e"),
    ("rw_save", "cw"), ("wwAvg_split", "cw"),
    ("rtheta_p_save", "c"), ("rho_p_save", "c"), ("theta_m_save", "c"), ("rr_save", "c"),
    ("rho_zz_old_split", "c"),
    ("scalars_init", "cs"), ("scalars_a", "cs"), ("scalars_b", "cs"),
    ("qtot", "c"), ("cqu_e", "e"),
    ("cqw", "cw"),
    ("cofrz", "L"),
    ("cofwr", "c"), ("cofwz", "c"), ("cofwt", "c"), ("a_tri", "c"), ("alpha_tri", "c"),
    ("gamma_tri", "c"),
    ("coftz", "cw"),
    ("tend_u", "e"), ("tend_u_euler", "e"), ("delsq_u", "e"),
    ("tend_w", "cw"), ("tend_w_euler", "cw"), ("tend_rw", "cw"), ("delsq_w", "cw"),
    ("tend_theta", "c"), ("tend_theta_euler", "c"), ("tend_rho", "c"), ("h_divergence", "c"),
    ("kdiff", "c"), ("dpdz", "c"), ("rthdynten", "c"), ("delsq_theta", "c"), ("delsq_div", "c"),
    ("delsq_vort", "v"),
    ("ru_p", "e"),
    ("rw_p", "cw"),
    ("rho_pp", "c"), ("rtheta_pp", "c"), ("rtheta_pp_old", "c"),
    ("ke_edge", "e"),
    ("ke_vertex", "v"), ("pv_vertex", "v"),
    ("pv_cell", "c"),
    ("hflux", "es"),
    ("flux_up", "es"), ("flux_tmp", "es"),
    ("s_max", "cs"), ("s_min", "cs"), ("scale_in", "cs"), ("scale_out", "cs"), ("rows", "cs"),
    ("wflux", "cws"),
    ("rho_int", "c"),
    ("flux_w_e", "e"), ("flux_th_e", "e"),
    ("ac_rs", "c"), ("ac_ts", "c"), ("ac_x", "cw"), ("b_tri", "c"), ("c_tri", "c"),
    ("tri_m", "c"), ("theta_edge_save", "e"), ("theta_edge_rsum", "e"),
)
# float32 members of mpasg_fields (after FIELDS, before status)
FIELDS32 = (
    ("u_f32", "e"), ("pv_edge_f32", "e"), ("flux_w_e_f32", "e"), ("flux_th_e_f32", "e"), ("ke_edge_f32", "e"),
    ("w_f32", "cw"), ("rw_f32", "cw"),
    ("theta_dev", "c"), ("theta_save_dev", "c"),
    ("pv_vertex_f32", "v"),
)
# float32 geometry copies of mpasg_mesh (after MESH_DBL_PTRS)
MESH_F32_PTRS = tuple(n + "_f32" for n in (
    "edgesOnCell_sign", "edgesOnVertex_sign", "dcEdge", "dvEdge", "invDcEdge", "invDvEdge", "invAreaCell",
    "invAreaTriangle", "kiteAreasOnVertex", "weightsOnEdge", "adv_coefs_p", "adv_coefs_m", "defc_a", "defc_b",
    "meshScalingDel2", "meshScalingDel4", "coeffs_reconstruct", "zxu", "zz", "rdzw", "rdzu", "fzm", "fzp", "fnm",
    "fnp", "rdnw"))

# float64 arrays appended after the float32 copies
MESH_TAIL_PTRS = ("zgrid", "u_init", "v_init", "angleEdge", "t_init", "cell_edge_geo", "cell_edge_sdv",
                  "cell_edge_es_w", "cell_edge_es_t", "edge_dcdv", "vertex_edge_sdc",
                  "cell_trig")


STAGE_NAMES = ("begin", "setup", "moist", "vert_imp_coefs", "dyn_tend_rk1", "dyn_tend",
               "smlstep_pert", "acoustic_step", "divergence_damping", "recover", "diagnostics",
               "split_bookkeeping", "scalars", "scalars_mono", "reconstruct")


class MeshStruct(C.Structure):
    _fields_ = ([(n, C.c_int32) for n in MESH_INT_DIMS] + [(n, C.c_double) for n in MESH_DOUBLES]
                + [(n, C.c_void_p) for n in MESH_INT_PTRS] + [(n, C.c_void_p) for n in MESH_DBL_PTRS]
                + [(n, C.c_void_p) for n in MESH_F32_PTRS] + [(n, C.c_void_p) for n in MESH_TAIL_PTRS])


CONFIG_MIXING_DOUBLES = ("h_theta_eddy_visc2", "v_mom_eddy_visc2", "v_theta_eddy_visc2", "mpas_cam_coef")
CONFIG_MIXING_INTS = ("number_cam_damping_levels", "scalar_advection_off")


CONFIG_DAMPING = (("rayleigh_damp_u_timescale_days", C.c_double), ("rayleigh_damp_u_levels", C.c_int32),
                  ("mix_perturbation", C.c_int32))


class ConfigStruct(C.Structure):
    _fields_ = ([(n, C.c_double) for n in CONFIG_DOUBLES] + [(n, C.c_int32) for n in CONFIG_INTS]
                + [(n, C.c_double) for n in CONFIG_MIXING_DOUBLES] + [(n, C.c_int32) for n in CONFIG_MIXING_INTS]
                + list(CONFIG_DAMPING))


class FieldsStruct(C.Structure):
    _fields_ = ([(n, C.c_void_p) for n, _ in FIELDS] + [(n, C.c_void_p) for n, _ in FIELDS32]
                + [("status", C.c_void_p)])


TRANSPOSE_PTRS = ("edgeCellSlot", "edgeVertexSlot", "eoeTransSlot", "cellsOnVertex", "vertexKite", "advPtr",
                  "advIdx")


class TransposeStruct(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in TRANSPOSE_PTRS]


EXPORTS = ("mpasg_abi_version", "mpasg_build_info", "mpasg_launch_count", "mpasg_prepare",
           "mpasg_step", "mpasg_step_timed",
           "mpasg_check_finite", "mpasg_moist_coefficients", "mpasg_vert_imp_coefs",
           "mpasg_dyn_tend", "mpasg_smlstep_pert", "mpasg_acoustic_step",
           "mpasg_divergence_damping", "mpasg_recover_large_step", "mpasg_solve_diagnostics",
           "mpasg_advance_scalars", "mpasg_advance_scalars_mono", "mpasg_reconstruct_2d",
           "mpasg_advance_scalars_static", "mpasg_numerics_check", "mpasg_surface_pressure",
           "mpasg_weighted_sq_sum", "mpasg_sfc_order", "mpasg_edge_order", "mpasg_permute_rows",
           "mpasg_tridiag_solve", "mpasg_tridiag_solve_vjp", "mpasg_tridiag_solve_jvp", "mpasg_tridiag_factor",
           "mpasg_tridiag_factor_vjp", "mpasg_tridiag_factor_jvp", "mpasg_autotune", "mpasg_fp64_peak",
           "mpasg_transport_vjp", "mpasg_transport_vjp_stage", "mpasg_step_taped", "mpasg_step_part",
           "mpasg_surface_pressure_vjp", "mpasg_surface_pressure_jvp", "mpasg_weighted_sq_sum_vjp",
           "mpasg_dyn_vjp_work_doubles", "mpasg_step_vjp_tape_doubles", "mpasg_vimp_vjp", "mpasg_dyn_tend_vjp",
           "mpasg_smlstep_vjp", "mpasg_acoustic_vjp", "mpasg_divdamp_vjp", "mpasg_recover_vjp", "mpasg_diag_vjp",
           "mpasg_step_vjp", "mpasg_prepare_vjp", "mpasg_step_tape", "mpasg_step_vjp_taped",
           "mpasg_prepare_derived", "mpasg_digest", "mpasg_step_jvp", "mpasg_prepare_jvp", "mpasg_vimp_jvp",
           "mpasg_dyn_tend_jvp", "mpasg_smlstep_jvp", "mpasg_acoustic_jvp", "mpasg_divdamp_jvp", "mpasg_recover_jvp", "mpasg_diag_jvp",
           "mpasg_step_vjp_window_tape_doubles", "mpasg_step_vjp_window")

# capacity of the library-owned edge scratch of mpasg_advance_scalars_static (float64 values)
STATIC_SCRATCH_DOUBLES = 1 << 22

_lib = None


def load() -> C.CDLL:
    """Load ``libmpasg.so`` once and declare the entry-point signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise MpasExtensionMissingError(
            f"{LIB_PATH} is missing: build it with mpas_dycore_pytorch_gb300.build.build() "
            "(the CUDA path has no CPU fallback)")
    lib = C.CDLL(str(LIB_PATH))
    P = C.POINTER
    m, c, f = P(MeshStruct), P(ConfigStruct), P(FieldsStruct)
    t = P(TransposeStruct)
    vp = C.c_void_p
    sig = {
        "mpasg_abi_version": ([], C.c_int),
        "mpasg_build_info": ([], C.c_char_p),
        "mpasg_launch_count": ([], C.c_longlong),
        "mpasg_step_timed": ([m, c, f, vp, vp, C.c_int, vp], C.c_int),
        "mpasg_prepare": ([m, c, f, vp, vp, vp, vp], C.c_int),
        "mpasg_prepare_derived": ([m, c, f, vp, vp, vp], C.c_int),
        "mpasg_digest": ([vp, C.c_longlong, vp, vp], C.c_int),
        "mpasg_step_jvp": ([m, c, f, f, vp, vp], C.c_int),
        "mpasg_step_vjp_window_tape_doubles": ([m, c, C.c_int], C.c_longlong),
        "mpasg_step_vjp_window": ([m, c, f, f, t, vp, vp, C.c_int, C.c_int, vp], C.c_int),
        "mpasg_prepare_jvp": ([m, c, f, f, vp, vp, vp], C.c_int),
        "mpasg_vimp_jvp": ([m, c, f, f, C.c_double, vp], C.c_int),
        "mpasg_dyn_tend_jvp": ([m, c, f, f, C.c_int, vp], C.c_int),
        "mpasg_smlstep_jvp": ([m, c, f, f, vp], C.c_int),
        "mpasg_acoustic_jvp": ([m, c, f, f, C.c_int, C.c_double, vp, vp], C.c_int),
        "mpasg_divdamp_jvp": ([m, c, f, f, C.c_double, vp], C.c_int),
        "mpasg_recover_jvp": ([m, c, f, f, C.c_int, C.c_int, C.c_double, vp], C.c_int),
        "mpasg_diag_jvp": ([m, c, f, f, C.c_int, vp], C.c_int),
        "mpasg_step": ([m, c, f, vp], C.c_int),
        "mpasg_check_finite": ([m, c, f, vp], C.c_int),
        "mpasg_moist_coefficients": ([m, c, f, vp], C.c_int),
        "mpasg_vert_imp_coefs": ([m, c, f, C.c_double, vp], C.c_int),
        "mpasg_dyn_tend": ([m, c, f, C.c_int, vp], C.c_int),
        "mpasg_smlstep_pert": ([m, c, f, vp], C.c_int),
        "mpasg_acoustic_step": ([m, c, f, C.c_int, C.c_double, vp], C.c_int),
        "mpasg_divergence_damping": ([m, c, f, C.c_double, vp], C.c_int),
        "mpasg_recover_large_step": ([m, c, f, C.c_int, C.c_int, C.c_double, vp], C.c_int),
        "mpasg_solve_diagnostics": ([m, c, f, C.c_int, vp], C.c_int),
        "mpasg_advance_scalars": ([m, c, f, C.c_int, C.c_double, vp], C.c_int),
        "mpasg_advance_scalars_mono": ([m, c, f, C.c_double, vp], C.c_int),
        "mpasg_reconstruct_2d": ([m, c, f, vp], C.c_int),
        "mpasg_advance_scalars_static": ([m, c, f, C.c_int, C.c_double, vp], C.c_int),
        "mpasg_numerics_check": ([C.c_int, vp, vp, C.c_longlong, vp], C.c_int),
        "mpasg_fp64_peak": ([vp, C.c_int, C.c_int, vp, vp], C.c_int),
        "mpasg_transport_vjp": ([m, c] + [vp] * 11, C.c_int),
        "mpasg_transport_vjp_stage": ([m, c, C.c_double, C.c_double, C.c_double] + [vp] * 12, C.c_int),
        "mpasg_step_taped": ([m, c, f, vp, vp], C.c_int),
        "mpasg_step_part": ([m, c, f, C.c_int, vp], C.c_int),
        "mpasg_surface_pressure": ([C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, C.c_double, vp, vp],
                                   C.c_int),
        "mpasg_weighted_sq_sum": ([C.c_longlong, vp, vp, vp, vp, vp], C.c_int),
        "mpasg_surface_pressure_vjp": ([C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, C.c_double] + [vp] * 6,
                                       C.c_int),
        "mpasg_surface_pressure_jvp": ([C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, C.c_double] + [vp] * 6,
                                       C.c_int),
        "mpasg_weighted_sq_sum_vjp": ([C.c_longlong] + [vp] * 7, C.c_int),
        "mpasg_sfc_order": ([C.c_longlong, vp, vp, vp, vp], C.c_int),
        "mpasg_edge_order": ([C.c_longlong, C.c_longlong, vp, vp, vp], C.c_int),
        "mpasg_permute_rows": ([vp, vp, vp, C.c_longlong, C.c_longlong, vp], C.c_int),
        "mpasg_autotune": ([m, c, f, vp, vp], C.c_int),
        "mpasg_tridiag_solve": ([C.c_longlong, C.c_int] + [vp] * 6, C.c_int),
        "mpasg_tridiag_solve_vjp": ([C.c_longlong, C.c_int] + [vp] * 11, C.c_int),
        "mpasg_tridiag_solve_jvp": ([C.c_longlong, C.c_int] + [vp] * 11, C.c_int),
        "mpasg_tridiag_factor": ([C.c_longlong, C.c_int] + [vp] * 6, C.c_int),
        "mpasg_tridiag_factor_vjp": ([C.c_longlong, C.c_int] + [vp] * 10, C.c_int),
        "mpasg_tridiag_factor_jvp": ([C.c_longlong, C.c_int] + [vp] * 10, C.c_int),
        "mpasg_dyn_vjp_work_doubles": ([m], C.c_longlong),
        "mpasg_step_vjp_tape_doubles": ([m, c], C.c_longlong),
        "mpasg_vimp_vjp": ([m, c, f, f, C.c_double, vp, vp], C.c_int),
        "mpasg_dyn_tend_vjp": ([m, c, f, f, t, C.c_int, vp, vp], C.c_int),
        "mpasg_smlstep_vjp": ([m, c, f, f, vp], C.c_int),
        "mpasg_acoustic_vjp": ([m, c, f, f, t, C.c_int, C.c_double, vp, vp], C.c_int),
        "mpasg_divdamp_vjp": ([m, c, f, f, C.c_double, vp, vp], C.c_int),
        "mpasg_recover_vjp": ([m, c, f, f, C.c_int, C.c_int, C.c_double, vp, vp], C.c_int),
        "mpasg_diag_vjp": ([m, c, f, f, t, C.c_int, vp, vp], C.c_int),
        "mpasg_step_vjp": ([m, c, f, f, t, vp, vp, vp], C.c_int),
        "mpasg_prepare_vjp": ([m, c, f, f, t] + [vp] * 7, C.c_int),
        "mpasg_step_tape": ([m, c, f, vp, vp], C.c_int),
        "mpasg_step_vjp_taped": ([m, c, f, f, t, vp, vp, vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.mpasg_abi_version() != ABI_VERSION:
        raise MpasExtensionMissingError("libmpasg.so ABI version mismatch; rebuild it")
    _lib = lib
    return lib


def check(rc: int, what: str) -> None:
    """Map a C status code to the package's exception types."""
    if rc >= 0:
        return
    if rc == -1:
        raise MpasConfigError(f"{what}: invalid argument (status {rc})")
    if rc == -3:
        raise MpasNumericalError(f"{what}: non-finite values (status {rc})")
    if rc == -5:
        raise MpasConfigError(
            f"{what}: nEdges * levels * scalars exceeds the library's static scratch of "
            f"{STATIC_SCRATCH_DOUBLES} values (status {rc}); use the entry point that takes "
            "caller scratch")
    raise MpasDeviceError(f"{what}: CUDA failure (status {rc})")
