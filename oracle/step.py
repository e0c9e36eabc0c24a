"""Oracle step driver: cold-start preparation and one split-explicit RK3 large step.

Restates the reference's orchestration of the stage functions in ``stages.py``:

* ``prepare``   -- ``atmosphere_model._prepare_timestep_state`` (atmosphere_model.py:782):
  coupled diagnostics (dynamics/init_coupled_diagnostics.py:147), padding sentinel
  (atmosphere_model.py:529), diagnostics with full tangential velocity
  (atmosphere_model.py:1186) and cell-wind reconstruction (:1339).
* ``srk3_step`` -- ``atm_srk3`` / ``_atm_srk3_impl`` (dynamics/time_integration.py:4897,
  :3420): ``atm_rk_integration_setup`` (:2497), 3 dynamics substeps x 3 RK stages of
  ``execute_rk_step`` (:5000), split bookkeeping (:3825-3942), the split transport RK3
  loop (:3954-4700) and the final reconstruction (:4729).
"""

from __future__ import annotations

import numpy as np

from . import stages as S

__all__ = ["Stepper", "rk_weights", "STAGE_NAMES", "COUPLED_STAGE_NAMES", "stage_names"]

RVORD = 461.6 / 287.0

STAGE_NAMES = {
    "moist": "mpas.moist_coefficients",
    "vimp": "mpas.vertical_implicit_coefficients_vert_imp_coefs",
    "dyn_tend": "mpas.dynamics_tendency_dyn_tend",
    "smlstep": "mpas.small_step_perturbation_smlstep_pert",
    "acoustic": "mpas.acoustic_step_acoustic_step",
    "divdamp": "mpas.divergence_damping",
    "recover": "mpas.large_step_recovery_recover_large_step",
    "diag": "mpas.diagnostic_solve_solve_diagnostics",
    "scalars": "mpas.explicit_scalar_transport_advance_scalars_transport",
    "scalars_mono": "mpas.monotonic_scalar_transport_advance_scalars_mono_transport",
    "reconstruct": "mpas.vector_reconstruction",
}
# the transport stages as the coupled mode calls them (inside the RK stages)
COUPLED_STAGE_NAMES = {
    "scalars": "mpas.explicit_scalar_transport_advance_scalars",
    "scalars_mono": "mpas.monotonic_scalar_transport_advance_scalars_mono",
}


def stage_names(key):
    """Every reference stage name under which ``key`` is called (split and coupled modes)."""
    return [STAGE_NAMES[key]] + ([COUPLED_STAGE_NAMES[key]] if key in COUPLED_STAGE_NAMES else [])


def rk_weights(dt, ns, order):
    """RK stage timesteps, acoustic substep timesteps and counts (time_integration.py:2787)."""
    if order == 3:
        rk_ts = [dt / 3.0, dt / 2.0, dt]
        rk_sub = [dt / 3.0, dt / ns, dt / ns]
        nsub = [1, max(ns // 2, 1), ns]
    else:
        rk_ts = [dt / 2.0, dt / 2.0, dt]
        rk_sub = [dt / ns, dt / ns, dt / ns]
        nsub = [max(ns // 2, 1), max(ns // 2, 1), ns]
    return rk_ts, rk_sub, nsub


class Stepper:
    """CPU restatement of the reference's large step on one padded state dict.

    ``mesh`` holds the static arrays and dimensions as the reference loader returns
    them (``ic_loader.load_initial_state``); ``config`` the validated namelist keys.
    ``on_stage(name, inputs, outputs)`` (optional) observes every stage call.
    """

    def __init__(self, mesh: dict, config: dict, on_stage=None):
        self.m = mesh
        self.cfg = dict(config)
        self.on_stage = on_stage
        m = mesh
        self.nc = int(m["nCells"])
        self.ne = int(m["nEdges"])
        self.nv = int(m["nVertices"])
        self.nl = int(m["nVertLevels"])
        self.dims = {"nCells": self.nc, "nEdges": self.ne, "nVertices": self.nv,
                     "nVertLevels": self.nl, "maxEdges": int(m["maxEdges"]),
                     "maxEdges2": int(m["maxEdges2"]), "vertexDegree": int(m["vertexDegree"])}
        self.order = int(self.cfg.get("config_time_integration_order", 3))
        self.ns = int(self.cfg.get("config_number_of_sub_steps", 2))
        # dynamics substeps per step; split transport off (or one substep) is the coupled
        # mode: scalars advance inside every RK stage (time_integration.py:1809-1878, 7890-7960)
        self.split = int(self.cfg.get("config_dynamics_split_steps", 3))
        if not bool(self.cfg.get("config_split_dynamics_transport", True)):
            self.split = 1
        self.coupled = self.split == 1
        self.epssm = float(self.cfg.get("config_epssm", 0.1))
        self.smdiv = float(self.cfg.get("config_smdiv", 0.1))
        self.len_disp = float(self.cfg.get("config_len_disp", 0.0))
        if self.len_disp <= 0.0:
            self.len_disp = float(np.min(m["dcEdge"][:self.ne]))
        # positive-definite selects the same limited last transport stage as monotonic
        # (time_integration.py:3979-3987); config_scalar_advection = false skips transport
        self.monotonic = bool(self.cfg.get("config_monotonic", True)) or \
            bool(self.cfg.get("config_positive_definite", False))
        self.advect = bool(self.cfg.get("config_scalar_advection", True))
        self.apvm = float(self.cfg.get("config_apvm_upwinding", 0.5))
        self.coef3 = float(m.get("coef_3rd_order", 0.25))
        self.c_s = float(m.get("c_s", 0.125))
        self.moist_start = int(m.get("moist_start", 1))
        self.moist_end = int(m.get("moist_end", 0))

    # ------------------------------------------------------------------ helpers
    def _call(self, key, fn, args):
        a = dict(self.m)
        a.update(self.dims)
        a.update(args)
        out = fn(a)
        if self.on_stage is not None:
            name = COUPLED_STAGE_NAMES[key] if self.coupled and key in COUPLED_STAGE_NAMES else STAGE_NAMES[key]
            self.on_stage(name, a, out)
        return out

    # ------------------------------------------------------------------ prepare
    def prepare(self, st: dict, dt: float) -> dict:
        """Cold-start preparation from loaded primitives (theta, rho, qv, u, w)."""
        m, nc, ne, nl = self.m, self.nc, self.ne, self.nl
        st = dict(st)
        zz = m["zz"][:nc]
        qv = st["qv"][:nc] if "qv" in st else np.zeros((nc, nl))
        theta_m = st["theta"][:nc] * (1.0 + RVORD * qv)
        rho_zz = st["rho"][:nc] / zz
        coe = S.idx0(m["cellsOnEdge"][:ne], nc)
        u = st["u"]
        rz_pad = np.concatenate([rho_zz, np.zeros((1, nl))])
        ru = 0.5 * u[:ne] * (rz_pad[coe[:, 0]] + rz_pad[coe[:, 1]])
        fzm, fzp = m["fzm"][:nl], m["fzp"][:nl]
        rho_i = fzp[None, 1:] * rho_zz[:, :nl - 1] + fzm[None, 1:] * rho_zz[:, 1:]
        zz_i = fzp[None, 1:] * zz[:, :nl - 1] + fzm[None, 1:] * zz[:, 1:]
        rw_int = st["w"][:nc, 1:nl] * rho_i * zz_i
        eoc = S.idx0(m["edgesOnCell"][:nc], ne)
        n_eoc = np.asarray(m["nEdgesOnCell"][:nc]).astype(np.int64)
        ru_pad = np.concatenate([ru, np.zeros((1, nl))])
        for j in range(eoc.shape[1]):
            valid = (j < n_eoc) & (eoc[:, j] < ne)
            e = np.where(valid, eoc[:, j], ne)
            flux = fzm[None, 1:] * ru_pad[e, 1:] + fzp[None, 1:] * ru_pad[e, :nl - 1]
            coef = m["zb_cell"][:nc, j, 1:nl] + S._sgn(flux) * m["zb3_cell"][:nc, j, 1:nl]
            c = m["edgesOnCell_sign"][:nc, j, None] * coef * flux * zz_i
            rw_int = rw_int - np.where(valid[:, None], c, 0.0)
        rw = np.zeros((nc + 1, nl + 1))
        rw[:nc, 1:nl] = rw_int
        rho_base = m["rho_base"][:nc]
        theta_base = m["theta_base"][:nc]
        rho_p = rho_zz - rho_base
        rtheta_base = theta_base * rho_base
        rtheta_p = theta_m * rho_p + rho_base * (theta_m - theta_base)
        rcv = S.RGAS / (S.CP - S.RGAS)
        exner = S.exner_pow(zz * (S.RGAS / S.P0) * (rtheta_p + rtheta_base), rcv)
        exner_base = S.exner_pow(zz * (S.RGAS / S.P0) * rtheta_base, rcv)
        pressure_p = zz * S.RGAS * (exner * rtheta_p + rtheta_base * (exner - exner_base))
        pressure_base = zz * S.RGAS * exner_base * rtheta_base

        def pc(x):
            o = np.zeros((nc + 1,) + x.shape[1:])
            o[:nc] = x
            return o

        st.update({"theta_m": pc(theta_m), "rho_zz": pc(rho_zz), "rho_p": pc(rho_p),
                   "rtheta_base": pc(rtheta_base), "rtheta_p": pc(rtheta_p), "exner": pc(exner),
                   "exner_base": pc(exner_base), "pressure_p": pc(pressure_p),
                   "pressure_base": pc(pressure_base), "rw": rw,
                   "ru": np.concatenate([ru, np.zeros((1, nl))])})
        st["rho_zz"][nc] = 1.0
        st.setdefault("rt_diabatic_tend", np.zeros((nc + 1, nl)))
        d = self._call("diag", S.solve_diagnostics,
                       {"u": st["u"], "h": st["rho_zz"], "v_in": None, "rk_step": 3, "dt": dt,
                        "config_apvm_upwinding": self.apvm})
        st.update(d)
        st["rho_edge"] = d["h_edge"]
        st.update(self._call("reconstruct", S.reconstruct_2d, {"u": st["u"]}))
        return st

    # ------------------------------------------------------------------ one large step
    def srk3_step(self, st: dict, dt: float) -> dict:
        m, nc, ne, nl = self.m, self.nc, self.ne, self.nl
        st = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
        split = self.split
        dt_dyn = dt / split
        rk_ts, rk_sub, nsub = rk_weights(dt_dyn, self.ns, self.order)
        epssm = self.epssm
        rcv = S.RGAS / (S.CP - S.RGAS)
        c2 = S.CP * rcv
        resm = (1.0 - epssm) / (1.0 + epssm)

        # atm_rk_integration_setup
        st["theta_m"][nc] = 0.0
        save = {"ru_save": st["ru"].copy(), "rw_save": st["rw"].copy(),
                "rtheta_p_save": st["rtheta_p"].copy(), "rho_p_save": st["rho_p"].copy(),
                "theta_m_save": st["theta_m"].copy(), "rr_save": st["rho_p"].copy()}
        rho_zz_old_split = st["rho_zz"].copy()
        scalars_init = st["scalars"].copy()
        ru_avg_split = np.zeros((ne + 1, nl))
        ww_avg_split = np.zeros((nc + 1, nl + 1))
        work = {"ru_p": np.zeros((ne + 1, nl)), "rw_p": np.zeros((nc + 1, nl + 1)),
                "rho_pp": np.zeros((nc + 1, nl)), "rtheta_pp": np.zeros((nc + 1, nl)),
                "rtheta_pp_old": np.zeros((nc + 1, nl)), "ruAvg": np.zeros((ne + 1, nl)),
                "wwAvg": np.zeros((nc + 1, nl + 1))}
        tend = {"tend_rho": np.zeros((nc + 1, nl))}
        zero_c = np.zeros(nc + 1)
        zero_e = np.zeros(ne + 1)

        moist = self._call("moist", S.moist_coefficients,
                           {"scalars": st["scalars"], "moist_start": self.moist_start,
                            "moist_end": self.moist_end})
        coefs = None
        for substep in range(1, split + 1):
            for rk in range(1, 4):
                dts = rk_sub[rk - 1]
                if rk == 1 or (rk == 2 and self.order == 3):
                    coefs = self._call("vimp", S.vert_imp_coefs, {
                        "dts": dts, "epssm": epssm, "gravity": S.GRAVITY, "rgas": S.RGAS,
                        "cp": S.CP, "cqw": moist["cqw"], "p": st["exner"], "t": st["theta_m"],
                        "rb": m["rho_base"], "rtb": st["rtheta_base"], "pb": st["exner_base"],
                        "rt": st["rtheta_p"], "qtot": moist["qtot"]})
                dt_args = {
                    "rk_step": rk, "dt": dt, "coef_3rd_order": self.coef3, "c_s": self.c_s,
                    "config_horiz_mixing": self.cfg.get("config_horiz_mixing", "2d_smagorinsky"),
                    "config_del4u_div_factor": float(self.cfg.get("config_del4u_div_factor", 10.0)),
                    "config_h_mom_eddy_visc4": float(self.cfg.get("config_h_mom_eddy_visc4", 0.0)),
                    "config_h_theta_eddy_visc4": float(self.cfg.get("config_h_theta_eddy_visc4", 0.0)),
                    "config_visc4_2dsmag": float(self.cfg.get("config_visc4_2dsmag", 0.05)),
                    "config_h_theta_eddy_visc2": float(self.cfg.get("config_h_theta_eddy_visc2", 0.0)),
                    "config_v_mom_eddy_visc2": float(self.cfg.get("config_v_mom_eddy_visc2", 0.0)),
                    "config_v_theta_eddy_visc2": float(self.cfg.get("config_v_theta_eddy_visc2", 0.0)),
                    "config_mpas_cam_coef": float(self.cfg.get("config_mpas_cam_coef", 0.0)),
                    "config_number_cam_damping_levels": int(self.cfg.get("config_number_cam_damping_levels", 4)),
                    "config_mix_full": bool(self.cfg.get("config_mix_full", True)),
                    "config_rayleigh_damp_u": bool(self.cfg.get("config_rayleigh_damp_u", False)),
                    "config_rayleigh_damp_u_timescale_days":
                        float(self.cfg.get("config_rayleigh_damp_u_timescale_days", 5.0)),
                    "config_number_rayleigh_damp_u_levels":
                        int(self.cfg.get("config_number_rayleigh_damp_u_levels", 6)),
                    "config_len_disp": self.len_disp,
                    "u": st["u"], "v": st["v"], "w": st["w"], "ru": st["ru"], "rw": st["rw"],
                    "ru_save": save["ru_save"], "rw_save": save["rw_save"],
                    "theta_m": st["theta_m"], "theta_m_save": save["theta_m_save"],
                    "rho_zz": st["rho_zz"], "rho_edge": st["rho_edge"], "exner": st["exner"],
                    "divergence": st["divergence"], "vorticity": st["vorticity"], "ke": st["ke"],
                    "pv_edge": st["pv_edge"], "pp": st["pressure_p"], "rr": st["rho_p"],
                    "rr_save": save["rr_save"], "rb": m["rho_base"],
                    "cqw": moist["cqw"], "cqu": moist["cqu"], "qtot": moist["qtot"],
                    "rt_diabatic_tend": st["rt_diabatic_tend"], "tend_rho_in": tend["tend_rho"]}
                if rk > 1:
                    dt_args.update({"kdiff_in": tend["kdiff"], "tend_u_euler_in": tend["tend_u_euler"],
                                    "tend_w_euler_in": tend["tend_w_euler"],
                                    "tend_theta_euler_in": tend["tend_theta_euler"]})
                tend.update(self._call("dyn_tend", S.dyn_tend, dt_args))
                tend_rw = self._call("smlstep", S.smlstep_pert,
                                     {"w_tend": tend["tend_w"], "u_tend": tend["tend_u"]})["w_tend"]
                pre = "_vertical_implicit_coefficients_"
                for small in range(1, nsub[rk - 1] + 1):
                    ac = self._call("acoustic", S.acoustic_step, {
                        "small_step": small, "dts": dts, "epssm": epssm, "c2": c2, "rcv": rcv,
                        "resm": resm, "rdts": 1.0 / dts, "cofrz": coefs["cofrz"],
                        **{k: v for k, v in coefs.items() if k.startswith(pre)},
                        "specZoneMaskCell": zero_c, "specZoneMaskEdge": zero_e,
                        "rho_zz": st["rho_zz"], "theta_m": save["theta_m_save"], "exner": st["exner"],
                        "cqu": moist["cqu"], "ru": st["ru"], "ru_save": save["ru_save"],
                        "rw": st["rw"], "rw_save": save["rw_save"], "w": st["w"],
                        "tend_ru": tend["tend_u"], "tend_rho": tend["tend_rho"],
                        "tend_rt": tend["tend_theta"], "tend_rw": tend_rw, **work})
                    for k in ("ru_p", "ruAvg", "rho_pp", "rtheta_pp", "rtheta_pp_old", "rw_p", "wwAvg"):
                        work[k] = ac[k]
                    work["ru_p"] = self._call("divdamp", S.divergence_damping, {
                        "dts": dts, "config_smdiv": self.smdiv, "config_len_disp": self.len_disp,
                        "specZoneMaskEdge": zero_e, "theta_m": save["theta_m_save"],
                        "rtheta_pp": work["rtheta_pp"], "rtheta_pp_old": work["rtheta_pp_old"],
                        "ru_p": work["ru_p"]})["ru_p"]
                rec = self._call("recover", S.recover_large_step, {
                    "rk_step": rk, "ns": nsub[rk - 1], "dt": rk_ts[rk - 1],
                    "cf1": float(m["cf1"]), "cf2": float(m["cf2"]), "cf3": float(m["cf3"]),
                    "rho_p_save": save["rho_p_save"], "rho_pp": work["rho_pp"],
                    "rtheta_p_save": save["rtheta_p_save"], "rtheta_pp": work["rtheta_pp"],
                    "rtheta_base": st["rtheta_base"], "rt_diabatic_tend": st["rt_diabatic_tend"],
                    "exner_base": st["exner_base"], "wwAvg": work["wwAvg"],
                    "rw_save": save["rw_save"], "rw_p": work["rw_p"], "ruAvg": work["ruAvg"],
                    "ru_save": save["ru_save"], "ru_p": work["ru_p"]})
                for k in ("rho_p", "rho_zz", "rtheta_p", "theta_m", "u", "ru", "w", "rw"):
                    st[k] = rec[k]
                st["rho_zz"][nc] = 1.0
                work["ruAvg"] = rec["ruAvg"]
                work["wwAvg"] = rec["wwAvg"]
                if rk == 3:
                    st["exner"] = rec["exner"]
                    st["pressure_p"] = rec["pressure_p"]
                if self.coupled and self.advect and scalars_init.shape[2] > 0:
                    st["scalars"] = self._transport_stage(rk, rk_ts[rk - 1], work["ruAvg"], work["wwAvg"],
                                                          scalars_init, st["scalars"], rho_zz_old_split,
                                                          st["rho_zz"], advance_density=0)
                d = self._call("diag", S.solve_diagnostics, {
                    "u": st["u"], "h": st["rho_zz"], "v_in": st["v"], "rk_step": rk, "dt": dt,
                    "config_apvm_upwinding": self.apvm})
                st.update(d)
                st["rho_edge"] = d["h_edge"]
            # split bookkeeping (atm_rk_dynamics_substep_finish)
            ru_avg_split = work["ruAvg"].copy() if substep == 1 else ru_avg_split + work["ruAvg"]
            ww_avg_split = work["wwAvg"].copy() if substep == 1 else ww_avg_split + work["wwAvg"]
            if substep < split:
                st["theta_m"][nc] = 0.0
                save.update({"ru_save": st["ru"].copy(), "rw_save": st["rw"].copy(),
                             "rtheta_p_save": st["rtheta_p"].copy(), "rho_p_save": st["rho_p"].copy(),
                             "theta_m_save": st["theta_m"].copy()})
                save["rr_save"] = save["rho_p_save"]
        inv = 1.0 / float(split)
        ru_avg = ru_avg_split * inv
        ww_avg = ww_avg_split * inv
        st["ruAvg"] = ru_avg
        st["wwAvg"] = ww_avg

        if not self.coupled and self.advect:
            # split transport RK3 with the substep-averaged mass fluxes
            scalars_new = scalars_init.copy()
            for rk in range(1, 4):
                # transport stage dts; the first is dt/2 for RK2 (time_integration.py:3366-3370)
                dt_t = [dt / 2.0 if self.order == 2 else dt / 3.0, dt / 2.0, dt][rk - 1]
                scalars_new = self._transport_stage(rk, dt_t, ru_avg, ww_avg, scalars_init, scalars_new,
                                                    rho_zz_old_split, st["rho_zz"], advance_density=1)
            st["scalars"] = scalars_new
        st.update(self._call("reconstruct", S.reconstruct_2d, {"u": st["u"]}))
        return st

    def _transport_stage(self, rk, dt_t, uh, ww, scalars_old, scalars_new, rho_old, rho_new, advance_density):
        """One transport RK stage: monotone at the last stage when config_monotonic, else
        explicit (time_integration.py:3954-4700 split, :7930-8200 coupled)."""
        if rk == 3 and self.monotonic:
            out = self._call("scalars_mono", S.advance_scalars_mono, {
                "dt": dt_t, "coef_3rd_order": self.coef3, "uhAvg": uh, "wwAvg": ww,
                "rho_zz_old": rho_old, "rho_zz_new": rho_new,
                "scalars_old": scalars_old, "scalars_new": scalars_new,
                "scalar_tend": np.zeros_like(scalars_old)})
            return out["scalars_new"]
        out = self._call("scalars", S.advance_scalars, {
            "rk_step": rk, "dt": dt_t, "coef_3rd_order": self.coef3,
            "config_time_integration_order": self.order, "advance_density": advance_density,
            "do_physics": False, "scalar_old": scalars_old, "scalar_new": scalars_new,
            "scalar_tend_save": np.zeros_like(scalars_old), "rho_zz_old": rho_old,
            "rho_zz_new": rho_new, "uhAvg": uh, "wwAvg": ww,
            "horiz_flux_arr": np.zeros((self.ne + 1, self.nl, scalars_old.shape[2]))})
        return out["scalar_new"]
