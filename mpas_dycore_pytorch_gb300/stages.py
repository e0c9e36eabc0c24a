"""Per-stage operators with the reference's keyword names (parity taps).

``run_stage(model, key, kwargs)`` copies the reference stage's keyword arrays into the
model's device fields, calls the matching C entry point and returns the stage outputs
under the reference's output names.  ``key`` is one of ``STAGES``; the reference function
each one replaces is listed beside it.
"""

from __future__ import annotations

import ctypes as C
from typing import Any, Mapping

import torch

from .device import _int

PRE = "_vertical_implicit_coefficients_"

# key: (C entry point, reference function, {ref input: field}, {ref output: field})
STAGES: dict[str, tuple[str, str, dict, dict]] = {
    "moist": ("mpasg_moist_coefficients", "dynamics/moist_coefficients.py:124",
              {"scalars": "scalars"}, {"qtot": "qtot", "cqw": "cqw", "cqu": "cqu_e"}),
    "vimp": ("mpasg_vert_imp_coefs", "dynamics/vert_imp_coefs.py:188",
             {"cqw": "cqw", "p": "exner", "t": "theta_m", "rtb": "rtheta_base", "pb": "exner_base",
              "rt": "rtheta_p", "qtot": "qtot"},
             {"cofrz": "cofrz", PRE + "cofwr_active": "cofwr", PRE + "cofwz_active": "cofwz",
              PRE + "coftz_active": "coftz", PRE + "cofwt_active": "cofwt",
              PRE + "a_tri_active": "a_tri", PRE + "alpha_tri_active": "alpha_tri",
              PRE + "gamma_tri_active": "gamma_tri"}),
    "dyn_tend": ("mpasg_dyn_tend", "dynamics/dyn_tend.py:10836",
                 {"u": "u", "v": "v", "w": "w", "ru": "ru", "rw": "rw", "ru_save": "ru_save",
                  "rw_save": "rw_save", "theta_m": "theta_m", "theta_m_save": "theta_m_save",
                  "rho_zz": "rho_zz", "rho_edge": "h_edge", "exner": "exner",
                  "divergence": "divergence", "vorticity": "vorticity", "ke": "ke",
                  "pv_edge": "pv_edge", "pp": "pressure_p", "rr": "rho_p", "rr_save": "rr_save",
                  "cqw": "cqw", "cqu": "cqu_e", "rt_diabatic_tend": "rt_diabatic_tend",
                  "qtot": "qtot", "tend_rho_in": "tend_rho", "kdiff_in": "kdiff",
                  "tend_u_euler_in": "tend_u_euler", "tend_w_euler_in": "tend_w_euler",
                  "tend_theta_euler_in": "tend_theta_euler"},
                 {"tend_u": "tend_u", "tend_rho": "tend_rho", "tend_theta": "tend_theta",
                  "tend_w": "tend_w", "tend_u_euler": "tend_u_euler", "tend_w_euler": "tend_w_euler",
                  "tend_theta_euler": "tend_theta_euler", "h_divergence": "h_divergence",
                  "kdiff": "kdiff", "rthdynten": "rthdynten"}),
    "smlstep": ("mpasg_smlstep_pert", "dynamics/smlstep_pert.py:373",
                {"w_tend": "tend_w", "u_tend": "tend_u"}, {"w_tend": "tend_rw"}),
    "acoustic": ("mpasg_acoustic_step", "dynamics/acoustic_step.py:1297",
                 {"rho_zz": "rho_zz", "theta_m": "theta_m_save", "exner": "exner", "rho_pp": "rho_pp",
                  "rtheta_pp": "rtheta_pp", "rtheta_pp_old": "rtheta_pp_old", "cqu": "cqu_e",
                  "ru": "ru", "ru_save": "ru_save", "ru_p": "ru_p", "ruAvg": "ruAvg",
                  "tend_ru": "tend_u", "tend_rho": "tend_rho", "tend_rt": "tend_theta", "w": "w",
                  "rw": "rw", "rw_save": "rw_save", "rw_p": "rw_p", "wwAvg": "wwAvg",
                  "tend_rw": "tend_rw", "cofrz": "cofrz", PRE + "cofwr_active": "cofwr",
                  PRE + "cofwz_active": "cofwz", PRE + "coftz_active": "coftz",
                  PRE + "cofwt_active": "cofwt", PRE + "a_tri_active": "a_tri",
                  PRE + "alpha_tri_active": "alpha_tri", PRE + "gamma_tri_active": "gamma_tri"},
                 {"ru_p": "ru_p", "ruAvg": "ruAvg", "rho_pp": "rho_pp", "rtheta_pp": "rtheta_pp",
                  "rtheta_pp_old": "rtheta_pp_old", "rw_p": "rw_p", "wwAvg": "wwAvg"}),
    "divdamp": ("mpasg_divergence_damping", "dynamics/divergence_damping.py:299",
                {"theta_m": "theta_m_save", "rtheta_pp": "rtheta_pp", "rtheta_pp_old": "rtheta_pp_old",
                 "ru_p": "ru_p"}, {"ru_p": "ru_p"}),
    "recover": ("mpasg_recover_large_step", "dynamics/recover_large_step.py:1090",
                {"rho_p_save": "rho_p_save", "rho_pp": "rho_pp", "rtheta_p_save": "rtheta_p_save",
                 "rtheta_pp": "rtheta_pp", "rtheta_base": "rtheta_base",
                 "rt_diabatic_tend": "rt_diabatic_tend", "exner_base": "exner_base",
                 "wwAvg": "wwAvg", "rw_save": "rw_save", "rw_p": "rw_p", "ruAvg": "ruAvg",
                 "ru_save": "ru_save", "ru_p": "ru_p"},
                {"w": "w", "rw": "rw", "wwAvg": "wwAvg", "rho_p": "rho_p", "rho_zz": "rho_zz",
                 "rtheta_p": "rtheta_p", "theta_m": "theta_m", "u": "u", "ru": "ru",
                 "ruAvg": "ruAvg", "exner": "exner", "pressure_p": "pressure_p"}),
    "diag": ("mpasg_solve_diagnostics", "dynamics/solve_diagnostics.py:1052",
             {"u": "u", "h": "rho_zz", "v_in": "v"},
             {"h_edge": "h_edge", "v": "v", "divergence": "divergence", "vorticity": "vorticity",
              "ke": "ke", "pv_edge": "pv_edge"}),
    "scalars": ("mpasg_advance_scalars", "dynamics/advance_scalars.py:1272",
                {"scalar_old": "scalars_init", "scalar_new": "scalars_a", "rho_zz_old": "rho_zz_old_split",
                 "rho_zz_new": "rho_zz", "uhAvg": "ruAvg", "wwAvg": "wwAvg"},
                {"scalar_new": "scalars_b"}),
    "scalars_mono": ("mpasg_advance_scalars_mono", "dynamics/advance_scalars_mono.py:2878",
                     {"scalars_old": "scalars_init", "scalars_new": "scalars_a", "uhAvg": "ruAvg",
                      "wwAvg": "wwAvg", "rho_zz_old": "rho_zz_old_split", "rho_zz_new": "rho_zz"},
                     {"scalars_new": "scalars_b"}),
    "reconstruct": ("mpasg_reconstruct_2d", "dynamics/vector_reconstruction.py:311",
                    {"u": "u"},
                    {"uReconstructX": "uReconstructX", "uReconstructY": "uReconstructY",
                     "uReconstructZ": "uReconstructZ", "uReconstructZonal": "uReconstructZonal",
                     "uReconstructMeridional": "uReconstructMeridional",
                     "ur_cell": "uReconstructZonal", "vr_cell": "uReconstructMeridional"}),
}


def _scalar_args(key: str, kw: Mapping[str, Any]) -> tuple:
    f = lambda n: C.c_double(float(kw[n]))
    i = lambda n: C.c_int(int(kw[n]))
    if key == "vimp":
        return (f("dts"),)
    if key == "dyn_tend":
        return (i("rk_step"),)
    if key == "acoustic":
        return (i("small_step"), f("dts"))
    if key == "divdamp":
        return (f("dts"),)
    if key == "recover":
        return (i("rk_step"), i("ns"), f("dt"))
    if key == "diag":
        return (i("rk_step"),)
    if key == "scalars":
        return (i("rk_step"), f("dt"))
    if key == "scalars_mono":
        return (f("dt"),)
    return ()


def run_stage(model, key: str, kwargs: Mapping[str, Any]) -> dict[str, torch.Tensor]:
    """Run one stage of ``model`` on reference-named inputs; returns reference-named outputs."""
    entry, _ref, inputs, outputs = STAGES[key]
    st = model.state
    for ref_name, field in inputs.items():
        if ref_name in kwargs and kwargs[ref_name] is not None and hasattr(kwargs[ref_name], "shape"):
            st.load({field: kwargs[ref_name]}, keys=(field,))
    model.call(entry, *_scalar_args(key, kwargs))
    torch.cuda.current_stream().synchronize()
    return {ref: st.f[field].clone() for ref, field in outputs.items()}
