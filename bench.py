"""Throughput of the GB300 MPAS large step, in cell-level-steps/s.

Default workload: the plain-float64 forecast on the level-6 icosahedral mesh (40962 cells,
122880 edges) with 55 levels to 30 km (lowest layer 50 m), 32 seeded theta bumps (seed 1),
3 passive tracers with the monotone limiter, dt = 720 s, split 3 x RK3 x 2 acoustic
substeps.  A "step" is one large step (``atm_srk3``).  Synthetic data of those shapes;
no dataset is involved.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

The GB300 arm prints one JSON line with the device-resident throughput (``value``), the
end-to-end throughput through the public API with host buffers (``e2e``), the stage time
breakdown, the roofline of the dominant stage, a CPU baseline (the numpy oracle on a bounded
sample) and the SM clocks sampled during the timed region.  ``--impl reference`` times the
CPU implementation (the oracle port of the reference's float64 algorithm) on the host
cores.  With N > 1 (torchrun) every rank runs an independent replica (the path does not
shard: replicas only) and the value is the sum over ranks.
"""

from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-level-steps/s fwd & VJP, mixed/batched vs plain FP64 on GB300 at stated error"
UNIT = "cell-level-steps/s"

WORKLOADS = {
    # headline: level-6 mesh, 55 stretched levels, 32 bumps, 3 monotone tracers, dt 720 s
    "c1": dict(spec=dict(level=6, nlev=55, dz_bottom=50.0, seed=1, n_bumps=32, n_tracers=3),
               config=dict(config_monotonic=True), dt=720.0,
               name="plain float64 forward, level-6 icosahedral mesh 40962 cells x 55 levels, "
                    "3 monotone tracers, dt 720 s, split 3 x RK3 x ns 2"),
    # level-5 mesh, 41 levels (the differentiation workload's mesh; profiling size: state > L2,
    # a few GB at most)
    "c2": dict(spec=dict(level=5, nlev=41, seed=2, n_bumps=8, n_tracers=3),
               config=dict(config_monotonic=True), dt=900.0,
               name="plain float64 forward, level-5 mesh 10242 cells x 41 levels, 3 monotone tracers, dt 900 s"),
    # large forward: level-8 mesh, 55 stretched levels, 128 bumps, 3 monotone tracers, dt 180 s;
    # the dissipation length is the mesh's own spacing (30 km), as MPAS sets it per mesh
    "c4": dict(spec=dict(level=8, nlev=55, dz_bottom=50.0, seed=3, n_bumps=128, n_tracers=3),
               config=dict(config_monotonic=True, config_len_disp=30000.0), dt=180.0,
               name="plain float64 forward, level-8 icosahedral mesh 655362 cells x 55 levels, "
                    "3 monotone tracers, dt 180 s, split 3 x RK3 x ns 2", cpu_baseline=False),
    # CPU-runnable case: level-4 mesh, 26 uniform levels, 8 bumps, 1 non-monotone tracer, dt 1800 s
    "c0": dict(spec=dict(level=4, nlev=26, seed=0, n_bumps=8, n_tracers=1),
               config=dict(config_monotonic=False), dt=1800.0,
               name="plain float64 forward, level-4 mesh 2562 cells x 26 levels, 1 tracer, dt 1800 s"),
}
# DRAM bytes (read + write) per call and cell-level of a float64 stage, from an ncu capture
# of the tendency stage on the level-5 mesh (10242 cells x 41 levels), scaled to the
# workload by its cell-levels
TRAFFIC_B_PER_CELL_LEVEL = {"dyn_tend": 542.7}
# executed float64 flops (2 per FMA) per call and cell-level of a float64 stage, averaged
# over a large step's calls, from an ncu count on the same level-5 x 41 case
FP64_FLOP_PER_CELL_LEVEL = {"dyn_tend": 607.3}
FP64_INST_PER_CELL_LEVEL = {"dyn_tend": 446.3}  # DFMA + DMUL + DADD issued
BASE_CFG = {"config_time_integration_order": 3, "config_len_disp": 120000.0,
            "config_number_of_sub_steps": 2, "config_dynamics_split_steps": 3}


def _cfg(w):
    c = dict(BASE_CFG)
    c.update(w["config"])
    c["config_dt"] = w["dt"]
    return c


# ------------------------------------------------------------------------------ CPU side
def _save_case(w):
    """The workload's loaded state and mesh, built once and written to a temporary .npz that
    the spawned oracle workers load (the level-6 mesh takes a while to generate); returns
    (path, loaded state)."""
    import numpy as np

    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.loader import load_case
    st, _ = load_case(CaseSpec(**w["spec"]), _cfg(w), as_torch=False)
    fd, path = tempfile.mkstemp(suffix=".npz")
    os.close(fd)
    arrays = {k: np.asarray(v) for k, v in st.items() if isinstance(v, (np.ndarray, int, float, np.integer, np.floating))}
    np.savez(path, **arrays)
    return path, st


# host memory one oracle process needs on the level-6 x 55 workload (peak RSS measured
# there: 7.8 GB including the case build); concurrent processes are capped by it
ORACLE_PROC_BYTES = {"c1": 8e9}


def _oracle_procs(w_key: str, want: int) -> int:
    """Concurrent oracle processes: at most one per core and as many as the host's
    available memory holds."""
    cores = max(1, os.cpu_count() or 1)
    try:
        avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    except (ValueError, OSError, AttributeError):
        avail = None
    by_mem = int(avail // ORACLE_PROC_BYTES.get(w_key, 2e9)) if avail else cores
    return max(1, min(want, cores, by_mem))


def _oracle_steps(args):
    """One worker: ``nsteps`` large steps of the oracle on the workload's own mesh from its
    prepared state (the preparation is untimed); returns (cell-levels, seconds)."""
    path, cfg, dt, nsteps = args
    sys.path.insert(0, str(ROOT))
    import numpy as np

    from oracle.step import Stepper
    z = np.load(path)
    st = {k: (z[k].item() if z[k].ndim == 0 else z[k]) for k in z.files}
    s = Stepper(st, cfg)
    prep = s.prepare(st, dt)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        prep = s.srk3_step(prep, dt)
    return nsteps * int(st["nCells"]) * int(st["nVertLevels"]), time.perf_counter() - t0


def cpu_throughput(w, procs: int, nsteps: int = 1, path: str | None = None):
    """Oracle throughput on the workload's own mesh: ``procs`` concurrent spawned processes,
    each timing ``nsteps`` large steps from the prepared state; the slowest bounds the wall
    time.  Returns (cell-levels, wall seconds)."""
    own = path is None
    path = path or _save_case(w)[0]
    try:
        ctx = mp.get_context("spawn")
        with ctx.Pool(procs) as pool:
            res = pool.map(_oracle_steps, [(path, _cfg(w), w["dt"], nsteps)] * procs)
    finally:
        if own:
            os.unlink(path)
    return sum(cl for cl, _ in res), max(sec for _, sec in res)


# ------------------------------------------------------------------------------ clocks
class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        try:
            for line in open(self.path):
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    mx = max(mx, float(p[2]))
                except ValueError:
                    continue
                for n, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        finally:
            os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def replica_throughput(ms_local: float, cell_levels_per_step: int, K: int, world: int, device=None):
    """Whole-job throughput of ``world`` independent replicas: the slowest rank's time
    (all-reduce MAX; no exchange otherwise) and the cell-level-steps of all ranks over it."""
    import torch
    ms = float(ms_local)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * cell_levels_per_step * K / (ms / 1e3)


def _time_steps(step, K, W):
    """ms per step of ``step()`` over K calls after W warm-up calls (CUDA events)."""
    import torch
    for _ in range(W):
        step()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(K):
        step()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / K


def _tune(model, args):
    """The autotuner, or a fixed tile (--tile 1/2/4: profiling runs, where ncu's serialised
    replay would distort the tuner's own timings)."""
    if args.tile == "auto":
        return model.autotune()
    model.cstruct.tile_tend_u = int(args.tile)
    model._graph = None
    return {"tend_u_levels_per_thread": int(args.tile), "tend_u_ms": None, "fixed": True}


def _graph_model(model):
    model.step()  # eager first step (shared-memory opt-ins happen before capture)
    model.capture_graph()
    return model


def measure_forms(args, dev, st, cfg, w, ms_plain):
    """The mixed form on the same workload and the batched ensemble of level-5 members
    (float64 and mixed), each timed like the headline (graph replay, CUDA events)."""
    import numpy as np
    import torch

    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.ensemble import Ensemble, member_cases

    K, W = args.steps, args.warmup
    S = int(st["scalars"].shape[-1])
    forms = {}
    # mixed form: throughput and its per-field error against float64 after 24 steps
    nerr = 24
    ends = {}
    for prec in ("float64", "mixed"):
        m = Model(st, cfg, w["dt"], num_scalars=S, device=dev, precision=prec, order=args.order)
        m.prepare(st)
        tune = _tune(m, args)
        _graph_model(m)
        for _ in range(nerr - 1):
            m.step()
        torch.cuda.synchronize()
        ends[prec] = {k: m.state.f[k][:-1].clone() for k in STATE_KEYS}
        if prec == "mixed":
            ms_mixed = _time_steps(m.step, K, W)
            timed = _timed_step_graph(m, m.lib, K)
            timed[0].replay()
            torch.cuda.synchronize()
            stage_ms, calls_per = _stage_ms(timed, K)
            roof_mixed = _stage_roofline(stage_ms, calls_per, S, int(st["nCells"]), int(st["nVertLevels"]),
                                         "mixed", dev)
            roof_mixed["bytes_model"] = ("v1 units weighted by width: u, pv_edge, w, rw read as float32 in "
                                         "dyn_tend, everything else float64")
            del timed
        del m
        torch.cuda.empty_cache()
    err = {}
    for k in STATE_KEYS:
        den = torch.linalg.vector_norm(ends["float64"][k]).item()
        if den > 0:
            err[k] = torch.linalg.vector_norm(ends["mixed"][k] - ends["float64"][k]).item() / den
    del ends
    cl = st_cells_levels(st)
    forms["mixed"] = {"value": cl / (ms_mixed / 1e3), "ms_per_step": ms_mixed,
                      "speedup_vs_float64": ms_plain / ms_mixed,
                      "max_rel_l2_vs_float64_after_24_steps": max(err.values()),
                      "worst_field": max(err, key=err.get), "dtype": "f32 stencils / f64 state",
                      "autotune": tune, "roofline": roof_mixed, "stage_ms_per_step": stage_ms}
    if args.ensemble > 0:
        ew = WORKLOADS["c2"]
        ecfg = _cfg(ew)
        spec = CaseSpec(**ew["spec"])
        single, _ = __import__("mpas_dycore_pytorch_gb300.loader", fromlist=["load_case"]).load_case(
            spec, ecfg, as_torch=False)
        m = Model(single, ecfg, ew["dt"], num_scalars=S, device=dev, order=args.order)
        m.prepare(single)
        _tune(m, args)
        ms_single = _time_steps(_graph_model(m).step, K, W)
        cl1 = st_cells_levels(single)
        del m
        torch.cuda.empty_cache()
        members = member_cases(spec, seeds=list(range(100, 100 + args.ensemble)), config=ecfg, u_noise=0.5)
        for prec in ("float64", "mixed"):
            ens = Ensemble(members, ecfg, ew["dt"], precision=prec, device=dev, order=args.order)
            etune = _tune(ens.model, args)
            _graph_model(ens.model)
            ms_e = _time_steps(ens.step, K, W)
            bad = ens.model.check_finite()
            forms["batched" if prec == "float64" else "batched_mixed"] = {
                "members": args.ensemble, "member_workload": ew["name"].replace("plain float64 forward, ", ""),
                "value": ens.cell_levels / (ms_e / 1e3), "ms_per_step": ms_e,
                "aggregate_vs_single_member_float64": (ens.cell_levels / ms_e) / (cl1 / ms_single),
                "single_member_float64_value": cl1 / (ms_single / 1e3), "nonfinite": bad,
                "state_bytes": ens.model.state.bytes, "autotune": etune}
            del ens
            torch.cuda.empty_cache()
    return forms


def measure_scalar_vjp(args, dev):
    """The scalar VJP (tracer_adjoint: taped forward + transposed transport, what
    run_simulation.vjp with track_keys=("scalars",) runs after its setup) on the level-5 x
    41 mesh (explicit transport, 3 passive tracers, 24 steps at dt 900 s), against the plain
    forward of the same 24 steps replayed from a CUDA graph; CUDA events on the stream."""
    import torch

    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.loader import load_case
    from mpas_dycore_pytorch_gb300.tracer_adjoint import ScalarTape, scalars_vjp, transport_adjacency

    w = WORKLOADS["c2"]
    cfg = dict(_cfg(w), config_monotonic=False)
    st, _ = load_case(CaseSpec(**w["spec"]), cfg, as_torch=False)
    nsteps = 24
    S = int(st["scalars"].shape[-1])
    m = Model(st, cfg, w["dt"], num_scalars=S, device=dev)
    m.prepare(st)
    m.step()
    m.capture_graph()
    ms_fwd = _time_steps(m.step, nsteps, args.warmup)
    del m
    torch.cuda.empty_cache()
    m = Model(st, cfg, w["dt"], num_scalars=S, device=dev)
    transport_adjacency(m.dmesh)  # host-built once per mesh
    g_end = torch.rand(m.state.f["scalars"].shape, dtype=torch.float64, device=dev)
    m.prepare(st)
    m.step()
    m.capture_graph()  # the taped forward replays the step graph (bitwise the eager step)
    ms = []
    for rep in range(2):  # the second repetition is timed
        m.prepare(st)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        tape = ScalarTape(m)
        for _ in range(nsteps):
            tape.step(m)
        g0 = scalars_vjp(m, tape, g_end)
        b.record()
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    cl = st_cells_levels(st)
    return {"workload": "level-5 mesh 10242 cells x 41 levels, 3 passive tracers, explicit transport, 24 steps",
            "value": cl * nsteps / (ms[-1] / 1e3), "unit": UNIT, "ms": ms[-1],
            "forward_graph_ms": ms_fwd * nsteps, "vjp_over_forward": ms[-1] / (ms_fwd * nsteps),
            "includes": "24 graph-replayed forward steps with the transport tape, then the transposed transport of "
                        "each step",
            "gradient_finite": bool(torch.isfinite(g0).all())}


DYN_VJP_SPEC = dict(level=5, nlev=41, seed=2, n_bumps=8, n_tracers=1, w_sine=0.1, round_wind_bits=16)


def measure_dynamics_vjp(args, dev):
    """The differentiation workload: gradient of the area-weighted squared surface-pressure
    anomaly after 24 steps (level-5 mesh 10242 cells x 41 levels, dt 900 s, 16-bit wind,
    0.1 m/s sinusoidal w) with respect to the initial u and theta, by the hand-written
    reverse mode (preparation, 24 steps with a checkpoint each, the objective's gradient, 24
    reverse steps each recomputing its step with the tape, the preparation's reverse), against
    the same 24 forward steps replayed from a CUDA graph; CUDA events on the stream.  Beside
    it: the same gradient with every step's tape kept (no recompute), the forward mode along
    a seeded direction with the JVP/VJP identity of the functional, and the mixed form's
    gradient against the float64 one."""
    import numpy as np
    import torch

    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure, surface_pressure_functional
    from mpas_dycore_pytorch_gb300.dyn_adjoint import DynamicsAdjoint, run_vjp
    from mpas_dycore_pytorch_gb300.loader import load_case

    cfg = dict(_cfg(WORKLOADS["c2"]), config_monotonic=False)
    dt, nsteps = 900.0, 24
    st, _ = load_case(CaseSpec(**DYN_VJP_SPEC), cfg, as_torch=False)
    nc = int(st["nCells"])
    m = Model(st, cfg, dt, num_scalars=1, device=dev)
    m.prepare(st)
    m.step()
    m.capture_graph()
    ms_fwd = _time_steps(m.step, nsteps, args.warmup)
    del m
    torch.cuda.empty_cache()
    m = Model(st, cfg, dt, num_scalars=1, device=dev)
    adj = DynamicsAdjoint(m)
    zz = torch.as_tensor(st["zz"], device=dev)
    zgrid = torch.as_tensor(st["zgrid"], device=dev)
    area = torch.as_tensor(st["areaCell"], device=dev)
    m.prepare(st)
    sp_ref = physics_interface_surface_pressure(
        nCells=nc, rho_zz=m.state.f["rho_zz"], zz=zz, qv=torch.zeros_like(m.state.f["rho_zz"]),
        pressure_p=m.state.f["pressure_p"], pressure_base=m.state.f["pressure_base"], zgrid=zgrid).detach().clone()

    def cotangents(final):
        rz = final["rho_zz"].detach().clone().requires_grad_(True)
        pp = final["pressure_p"].detach().clone().requires_grad_(True)
        sp = physics_interface_surface_pressure(nCells=nc, rho_zz=rz, zz=zz, qv=torch.zeros_like(rz), pressure_p=pp,
                                                pressure_base=final["pressure_base"], zgrid=zgrid)
        J = surface_pressure_functional(sp, sp_ref, area, nc)
        g_rz, g_pp = torch.autograd.grad(J, [rz, pp])
        return {"rho_zz": g_rz, "pressure_p": g_pp}

    def timed(mode):
        ms = []
        for rep in range(2):  # the second repetition is timed
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            grads, _ = run_vjp(m, st, nsteps, cotangents, adj, checkpoint=mode)
            b.record()
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return ms[-1], grads

    ms_none, g_none = timed("none")
    ms_step, grads = timed("step")
    same = all(bool(torch.equal(g_none[k], grads[k])) for k in ("u", "theta"))
    # forward mode along a seeded direction of u and theta (preparation and 24 steps of
    # values and tangents), and the JVP/VJP identity of the functional along it
    from mpas_dycore_pytorch_gb300.dyn_adjoint import DynamicsTangent, run_jvp
    tan = DynamicsTangent(m)
    rng = np.random.default_rng(2)
    pert = {}
    for k, scale in (("u", 1.0), ("theta", 0.1)):
        x = rng.standard_normal(tuple(np.asarray(st[k]).shape)) * scale
        x[-1] = 0.0
        pert[k] = torch.as_tensor(x)
    ms_jvp = []
    for rep in range(2):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        tans = run_jvp(m, st, nsteps, pert, tan)
        b.record()
        torch.cuda.synchronize()
        ms_jvp.append(a.elapsed_time(b))
    final = {k: v for k, v in m.export().items()}
    g_out = cotangents(final)
    dj_fwd = sum(float((g_out[k] * tans[k]).sum()) for k in g_out)
    dj_rev = sum(float((grads[k][:-1].cpu() * pert[k][:-1]).sum()) for k in pert)
    del tan
    torch.cuda.empty_cache()
    # the mixed form's gradient (its trajectory, linearised in float64) against the float64 one
    cfg_mixed = dict(cfg, config_precision="mixed")
    mm = Model(st, cfg_mixed, dt, num_scalars=1, device=dev)
    adj_m = DynamicsAdjoint(mm)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g_mixed, _ = run_vjp(mm, st, nsteps, cotangents, adj_m, checkpoint="none")
    a.record()
    g_mixed, _ = run_vjp(mm, st, nsteps, cotangents, adj_m, checkpoint="none")
    b.record()
    torch.cuda.synchronize()
    ms_mixed = a.elapsed_time(b)
    mixed_err = {k: float(torch.linalg.norm(g_mixed[k][:-1] - grads[k][:-1]) / torch.linalg.norm(grads[k][:-1]))
                 for k in ("u", "theta")}
    del mm, adj_m
    torch.cuda.empty_cache()
    ms = [ms_step]
    cl = st_cells_levels(st)
    finite = all(bool(torch.isfinite(grads[k]).all()) for k in ("u", "theta"))
    return {"workload": "level-5 mesh 10242 cells x 41 levels, dry, 16-bit wind, 0.1 m/s sinusoidal w, 24 steps at "
                        "dt 900 s; gradient of the area-weighted squared surface-pressure anomaly w.r.t. initial u and "
                        "theta",
            "value": cl * nsteps / (ms[-1] / 1e3), "unit": UNIT, "ms": ms[-1],
            "forward_graph_ms": ms_fwd * nsteps, "vjp_over_forward": ms[-1] / (ms_fwd * nsteps),
            "includes": "preparation, 24 eager forward steps with a checkpoint each, the objective's gradient, 24 "
                        "reverse steps (each recomputes its step with the tape), the preparation's reverse",
            "tape_bytes": int(adj.tape.numel() * 8) if adj.tape is not None else 0,
            "gradient_finite": finite,
            "no_recompute": {"ms": ms_none, "vjp_over_forward": ms_none / (ms_fwd * nsteps),
                             "value": cl * nsteps / (ms_none / 1e3), "tape_bytes": adj.tape_doubles() * 8 * nsteps,
                             "includes": "every step's tape kept from the forward pass (checkpoint_timesteps=False); "
                                         "the forward advances the dynamics only",
                             "same_gradient_bitwise": same},
            "jvp": {"ms": ms_jvp[-1], "jvp_over_forward": ms_jvp[-1] / (ms_fwd * nsteps),
                    "includes": "preparation and its tangent, 24 steps of the dynamics with their tangents (eager)",
                    "identity_rel": abs(dj_fwd - dj_rev) / abs(dj_rev)},
            "mixed": {"ms": ms_mixed, "vjp_over_forward": ms_mixed / (ms_fwd * nsteps),
                      "gradient_rel_l2_vs_float64": mixed_err,
                      "includes": "the mixed form's trajectory taped (checkpoint_timesteps=False), the reverse pass in "
                                  "float64"}}


def measure_large_vjp(args, dev, st, cfg, w, nsteps=12):
    """The large workload's gradient (level-8 mesh 655362 cells x 55 levels, dt 180 s): the
    area-weighted squared surface-pressure anomaly after 12 steps with respect to the initial
    u and theta, by the reverse mode with sqrt(N) step checkpoints and one dynamics substep
    taped at a time (checkpoint="sqrt"), in the mixed form and in float64; the dry dynamics
    do not read the scalars, so the models hold none.  Reports the time, the peak device
    memory, the mixed gradient's error against the float64 one, and a forward step of each
    form (CUDA graph) for the ratio."""
    import numpy as np
    import torch

    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure, surface_pressure_functional
    from mpas_dycore_pytorch_gb300.dyn_adjoint import DynamicsAdjoint, run_vjp

    nc = int(st["nCells"])
    zz = torch.as_tensor(st["zz"], device=dev)
    zgrid = torch.as_tensor(st["zgrid"], device=dev)
    area = torch.as_tensor(st["areaCell"], device=dev)
    out, grads = {}, {}
    for prec in ("mixed", "float64"):
        c = dict(cfg, config_precision=prec)
        m = Model(st, c, w["dt"], num_scalars=0, device=dev)
        m.prepare(st)
        m.step()
        m.capture_graph()
        fwd_ms = _time_steps(m.step, 3, 1)
        m.prepare(st)
        sp_ref = physics_interface_surface_pressure(
            nCells=nc, rho_zz=m.state.f["rho_zz"], zz=zz, qv=torch.zeros_like(m.state.f["rho_zz"]),
            pressure_p=m.state.f["pressure_p"], pressure_base=m.state.f["pressure_base"], zgrid=zgrid).detach().clone()

        def cotangents(final):
            rz = final["rho_zz"].detach().clone().requires_grad_(True)
            pp = final["pressure_p"].detach().clone().requires_grad_(True)
            sp = physics_interface_surface_pressure(nCells=nc, rho_zz=rz, zz=zz, qv=torch.zeros_like(rz),
                                                    pressure_p=pp, pressure_base=final["pressure_base"], zgrid=zgrid)
            g_rz, g_pp = torch.autograd.grad(surface_pressure_functional(sp, sp_ref, area, nc), [rz, pp])
            return {"rho_zz": g_rz, "pressure_p": g_pp}

        adj = DynamicsAdjoint(m)
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats(dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        g, _ = run_vjp(m, st, nsteps, cotangents, adj, checkpoint="sqrt")
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        grads[prec] = {k: g[k][:-1].cpu() for k in ("u", "theta")}
        out[prec] = {"ms": ms, "forward_graph_ms_per_step": fwd_ms, "vjp_over_forward": ms / (nsteps * fwd_ms),
                     "peak_device_gb": torch.cuda.max_memory_allocated(dev) / 1e9,
                     "window_tape_gb": adj.window_tape.numel() * 8 / 1e9 if adj.window_tape is not None else 0.0,
                     "gradient_finite": all(bool(torch.isfinite(g[k]).all()) for k in ("u", "theta"))}
        del m, adj, g
        torch.cuda.empty_cache()
    out["mixed"]["gradient_rel_l2_vs_float64"] = {
        k: float(np.linalg.norm((grads["mixed"][k] - grads["float64"][k]).numpy()) /
                 np.linalg.norm(grads["float64"][k].numpy())) for k in ("u", "theta")}
    out["workload"] = (f"level-8 mesh {nc} cells x {int(st['nVertLevels'])} levels, dry dynamics, {nsteps} steps at "
                       f"dt {w['dt']} s; gradient of the area-weighted squared surface-pressure anomaly w.r.t. initial "
                       f"u and theta; sqrt(N) step checkpoints, one dynamics substep taped at a time")
    return out


def profile_dynamics_vjp(dev, pairs=2):
    """For kernel profiles (ncu): the differentiation workload prepared, then ``pairs`` times
    one taped forward step (mpasg_step_tape) and one reverse step (mpasg_step_vjp_taped)
    from the prepared state.  Prints the CUDA-event times of the last pair; no bench line."""
    import torch

    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.dyn_adjoint import DynamicsAdjoint
    from mpas_dycore_pytorch_gb300.loader import load_case

    cfg = dict(_cfg(WORKLOADS["c2"]), config_monotonic=False)
    st, _ = load_case(CaseSpec(**DYN_VJP_SPEC), cfg, as_torch=False)
    m = Model(st, cfg, 900.0, num_scalars=1, device=dev)
    adj = DynamicsAdjoint(m)
    m.prepare(st)
    ck = adj.checkpoint()
    tape = torch.empty(adj.tape_doubles(), dtype=torch.float64, device=dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    for _ in range(int(pairs)):
        adj.restore(ck)
        adj.zero_cotangents()
        torch.cuda.synchronize()
        ev[0].record()
        adj.step_tape(tape)
        ev[1].record()
        adj.step_vjp_taped(tape)
        ev[2].record()
        torch.cuda.synchronize()
    print(f"taped forward {ev[0].elapsed_time(ev[1]):.3f} ms, reverse {ev[1].elapsed_time(ev[2]):.3f} ms")


def measure_ensemble_groups(args, dev):
    """The two-grid mixed-precision ensemble: 96 members of 10242 cells x 41 levels (dt
    900 s) and 32 members of 40962 cells x 55 stretched levels (dt 720 s), 2 monotone
    tracers, seeds 100-227 with u noise 0.5 m/s, all replayed from one CUDA graph.  Also
    times each member shape alone in float64 (the sequential baseline) and checks the
    first member of each group against its float64 solo run after 24 steps."""
    import torch

    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.ensemble import EnsembleGroups, member_cases

    K, W, nerr = args.steps, args.warmup, 24
    shapes = [("c2", 96, list(range(100, 196))), ("c1", 32, list(range(196, 228)))]
    groups, solo_ms, firsts = [], [], []
    for key, n, seeds in shapes:
        w = WORKLOADS[key]
        spec = CaseSpec(**dict(w["spec"], n_tracers=2))
        cfg = _cfg(w)
        mem = member_cases(spec, seeds=seeds[:n], config=cfg, u_noise=0.5)
        groups.append((mem, cfg, w["dt"]))
        firsts.append((mem[0], cfg, w["dt"]))
    # float64 solo runs of each group's first member: sequential baseline and error reference
    ref_end = []
    for m0, cfg, dt in firsts:
        solo = Model(m0, cfg, dt, num_scalars=2, device=dev, order=args.order)
        solo.prepare(m0)
        _tune(solo, args)
        solo.capture_graph()
        for _ in range(nerr):
            solo.step()
        torch.cuda.synchronize()
        exp = solo.export()  # the member's own order (the solo run may be in curve order)
        ref_end.append({k: exp[k][:-1] for k in STATE_KEYS})
        solo_ms.append(_time_steps(solo.step, K, W))
        del solo
        torch.cuda.empty_cache()
    ens = EnsembleGroups(groups, precision="mixed", device=dev, order=args.order)
    tune = [_tune(g.model, args) for g in ens.groups]
    ens.capture_graph()
    for _ in range(nerr):
        ens.step()
    torch.cuda.synchronize()
    err = {}
    for gi, ref in enumerate(ref_end):
        got = ens.member_state(gi, 0)
        for k, r in ref.items():
            den = torch.linalg.vector_norm(r).item()
            if den > 0:
                e = torch.linalg.vector_norm(got[k][:-1] - r).item() / den
                err[f"{shapes[gi][0]}:{k}"] = e
    ms = _time_steps(ens.step, K, W)
    seq_ms = sum(n * t for (_, n, _), t in zip(shapes, solo_ms))
    out = {"members": [n for _, n, _ in shapes],
           "member_workloads": ["10242 cells x 41 levels, dt 900 s", "40962 cells x 55 levels, dt 720 s"],
           "value": ens.cell_levels / (ms / 1e3), "ms_per_step": ms,
           "sequential_float64_ms_per_step": seq_ms, "speedup_vs_sequential_float64": seq_ms / ms,
           "max_rel_l2_first_members_vs_float64_after_24_steps": max(err.values()),
           "worst_field": max(err, key=err.get), "nonfinite": ens.check_finite(),
           "state_bytes": ens.state_bytes, "autotune": tune, "graph": "one graph, one stream per group"}
    del ens
    torch.cuda.empty_cache()
    return out


def fp64_roofline(flops_per_launch, inst_per_launch, launch_ms, dev):
    """{"achieved", "peak", "unit": "TFLOP/s", "frac"} for a float64-bound stage; the peak
    from mpasg_fp64_peak (1216 blocks x 256 threads x 4096 rounds of 8 FMAs).  A DMUL or
    DADD occupies the pipe like a DFMA but counts one flop, so "pipe_frac" (issued float64
    instructions against peak / 2 per second) is the utilisation of the bounding unit."""
    import ctypes as C

    import torch

    from mpas_dycore_pytorch_gb300 import _lib
    blocks = 152 * 8
    buf = torch.rand(blocks * 256, dtype=torch.float64, device=dev) * 0.5
    peak = C.c_double(0.0)
    rc = _lib.load().mpasg_fp64_peak(C.c_void_p(buf.data_ptr()), blocks, 4096, C.byref(peak),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "mpasg_fp64_peak")
    achieved = flops_per_launch / (launch_ms / 1e3) / 1e12
    pk = peak.value / 1e12
    pipe = inst_per_launch / (launch_ms / 1e3) / (peak.value / 2.0)
    return {"achieved": round(achieved, 4), "peak": round(pk, 4), "unit": "TFLOP/s", "frac": round(achieved / pk, 4),
            "pipe_frac": round(pipe, 4), "flops_per_launch": round(flops_per_launch),
            "fp64_instructions_per_launch": round(inst_per_launch),
            "peak_source": "measured in this run (mpasg_fp64_peak)",
            "flops_source": "ncu executed float64 instructions (2 flops per FMA), level-5 count scaled by cell-levels"}


def st_cells_levels(st):
    import numpy as np
    return int(np.asarray(st["nCells"]).reshape(-1)[0]) * int(np.asarray(st["nVertLevels"]).reshape(-1)[0])


def _timed_step_graph(model, lib, K, n_b=128):
    """One CUDA graph of K large steps through the library's timed step
    (mpasg_step_timed), which records an event at every stage boundary.  Returns (graph,
    events, stage kinds, event counts); replay it, then read the stages with _stage_ms."""
    import ctypes as C

    import torch
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(n_b)] for _ in range(K)]
    for row in evs:
        for e in row:
            e.record()  # materialise the cudaEvent_t
    torch.cuda.synchronize()
    ptrs = [(C.c_void_p * n_b)(*[C.c_void_p(e.cuda_event) for e in row]) for row in evs]
    kinds = [(C.c_int32 * n_b)() for _ in range(K)]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    counts = []
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            for k in range(K):
                counts.append(lib.mpasg_step_timed(C.byref(model.dmesh.struct), C.byref(model.cstruct),
                                                   C.byref(model.state.struct), ptrs[k], kinds[k], n_b,
                                                   C.c_void_p(s.cuda_stream)))
    torch.cuda.current_stream().wait_stream(s)
    if min(counts) < 0:
        raise RuntimeError(f"timed step failed: {counts}")
    return g, evs, kinds, counts, n_b


def _stage_ms(timed, K):
    """ms per step of every stage and calls per step, from a replayed _timed_step_graph."""
    from mpas_dycore_pytorch_gb300 import _lib
    _, evs, kinds, counts, n_b = timed
    stage_ms, stage_calls = {}, {}
    for k in range(K):
        for i in range(1, min(counts[k], n_b)):
            name = _lib.STAGE_NAMES[kinds[k][i]]
            stage_ms[name] = stage_ms.get(name, 0.0) + evs[k][i - 1].elapsed_time(evs[k][i])
            stage_calls[name] = stage_calls.get(name, 0) + 1
    stage_ms = {k: v / K for k, v in sorted(stage_ms.items(), key=lambda kv: -kv[1])}
    return stage_ms, {k: v // K for k, v in stage_calls.items()}


def _stage_roofline(stage_ms, calls_per, S, C_, L_, precision, dev):
    """HBM roofline of the dominant stage: the byte model's algorithmic bytes per call (every
    distinct input read and output written once, float64 units) over the stage's measured
    time per call; for the float64 form also its float64-pipe roofline."""
    from mpas_dycore_pytorch_gb300.bytes_model import stage_bytes_per_call
    peak, peak_kind = measured_peak_hbm()
    merged = dict(stage_ms)
    merged["dyn_tend"] = merged.pop("dyn_tend", 0.0) + merged.pop("dyn_tend_rk1", 0.0)
    merged["acoustic_divdamp"] = merged.pop("acoustic_step", 0.0) + merged.pop("divergence_damping", 0.0)
    calls = dict(calls_per)
    calls["dyn_tend"] = calls.get("dyn_tend", 0) + calls.get("dyn_tend_rk1", 0)
    calls["acoustic_divdamp"] = calls.get("acoustic_step", 0)
    keymap = {"vert_imp_coefs": "vert_imp_coefs", "dyn_tend": "dyn_tend", "smlstep_pert": "smlstep_pert",
              "acoustic_divdamp": "acoustic_divdamp", "recover": "recover", "diagnostics": "diagnostics"}
    dom = max((k for k in merged if k in keymap), key=lambda k: merged[k])
    per_call_ms = merged[dom] / max(calls[dom], 1)
    bytes_call = stage_bytes_per_call(keymap[dom], S, C_, L_, precision=precision)
    achieved = bytes_call / (per_call_ms / 1e3) / 1e9
    traffic = None
    if dom in TRAFFIC_B_PER_CELL_LEVEL and precision == "float64":
        traffic = round(TRAFFIC_B_PER_CELL_LEVEL[dom] * C_ * L_)
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": f"stage:{dom}",
            "peak_source": peak_kind, "algorithmic_bytes_per_launch": bytes_call,
            "launch_ms": round(per_call_ms, 4)}
    # the float64 form's real bound: the float64 pipe (GB300 runs float64 at 1/64 of
    # float32).  Executed float64 flops of the stage from an ncu count, against the
    # float64 peak measured here with the library's own multiply-add kernel.
    if dom in FP64_FLOP_PER_CELL_LEVEL and precision == "float64":
        roof["fp64_pipe"] = fp64_roofline(FP64_FLOP_PER_CELL_LEVEL[dom] * C_ * L_,
                                          FP64_INST_PER_CELL_LEVEL[dom] * C_ * L_, per_call_ms, dev)
    return roof


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------------------ GPU arm
def run_gb300(args, rank, world):
    import ctypes as C

    import numpy as np
    import torch

    from mpas_dycore_pytorch_gb300 import _lib
    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.bytes_model import bytes_per_cell_level_step
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.loader import load_case

    w = WORKLOADS[args.workload]
    cfg = _cfg(w)
    # the CPU baseline: one large step of the oracle on this workload, in a process spawned
    # before any CUDA work that runs while the GPU is measured (one host core of 16)
    cpu_job = None
    # (none on the level-8 workload: one step of the oracle there takes most of an hour)
    if rank == 0 and world == 1 and not args.no_cpu_baseline and w.get("cpu_baseline", True):
        case_path, st = _save_case(w)
        cpu_pool = mp.get_context("spawn").Pool(1)
        cpu_job = cpu_pool.apply_async(_oracle_steps, ((case_path, cfg, w["dt"], 1),))
    else:
        st, _ = load_case(CaseSpec(**w["spec"]), cfg, as_torch=False)
    torch.cuda.set_device(rank % torch.cuda.device_count())
    dev = torch.device("cuda", torch.cuda.current_device())
    S = int(st["scalars"].shape[-1])
    model = Model(st, cfg, w["dt"], num_scalars=S, device=dev, precision=args.precision, order=args.order)
    model.prepare(st)
    tuning = _tune(model, args)
    C_, L_ = model.dmesh.nCells, model.dmesh.nVertLevels
    lib = model.lib
    # launches per step (eager step, counted by the library)
    n0 = lib.mpasg_launch_count()
    model.step()
    torch.cuda.synchronize()
    launches_per_step = int(lib.mpasg_launch_count() - n0)

    # timed graph: K steps with stage-boundary events
    K, W = args.steps, args.warmup
    model.capture_graph()
    for _ in range(W):
        model.step()
    torch.cuda.synchronize()

    stage_ms = None
    timed = None
    try:
        timed = _timed_step_graph(model, lib, K)
    except Exception as exc:  # fall back to the plain graph; no stage breakdown
        print(f"[bench] stage-event graph unavailable: {exc}", file=sys.stderr)

    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clocks:
        start.record()
        if timed is not None:
            timed[0].replay()
        else:
            for _ in range(K):
                model.step()
        end.record()
        torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    ms, value = replica_throughput(ms, C_ * L_, K, world, dev)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    bad = model.check_finite()

    if timed is not None:
        stage_ms, calls_per = _stage_ms(timed, K)

    # roofline of the dominant stage
    roof = _stage_roofline(stage_ms, calls_per, S, C_, L_, args.precision, dev) if stage_ms else None

    # end to end through the public API with pinned host buffers
    keys = [k for k in STATE_KEYS]
    host = {k: torch.empty(model.state.f[k].shape, dtype=torch.float64, pin_memory=True) for k in keys}
    ex0 = model.export(clone=False)
    for k in keys:
        host[k].copy_(ex0[k])
    h2d = sum(t.numel() * 8 for t in host.values())
    # the two parts of a step as graphs; warm the host path (staging buffers, copy streams)
    model.capture_graph_parts()
    model.run_host(host, W)
    torch.cuda.synchronize()
    e_start = torch.cuda.Event(enable_timing=True)
    e_end = torch.cuda.Event(enable_timing=True)
    e_start.record()
    model.run_host(host, K)
    e_end.record()
    torch.cuda.synchronize()
    e_ms, e_value = replica_throughput(e_start.elapsed_time(e_end), C_ * L_, K, world, dev)
    e2e = {"value": e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": h2d}

    state_bytes = model.state.bytes
    forms = None
    if world == 1 and not args.no_forms and args.precision == "float64" and args.workload == "c1":
        del model, host
        torch.cuda.empty_cache()
        forms = measure_forms(args, dev, st, cfg, w, ms / K)
        forms["vjp_scalars"] = measure_scalar_vjp(args, dev)
        torch.cuda.empty_cache()
        forms["vjp_dynamics"] = measure_dynamics_vjp(args, dev)
        if args.ensemble_groups:
            forms["batched_two_grids"] = measure_ensemble_groups(args, dev)
    elif world == 1 and not args.no_forms and args.workload == "c4":
        del model, host
        torch.cuda.empty_cache()
        forms = {"vjp_sqrt_checkpointed": measure_large_vjp(args, dev, st, cfg, w)}

    cpu = None
    if cpu_job is not None:
        cl, wall = cpu_job.get()
        cpu_pool.close()
        cpu_pool.join()
        os.unlink(case_path)
        cpu = {"value": cl / wall, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"one large step of the numpy oracle on this workload's own mesh and options "
                         f"({cl} cell-levels) from its prepared state, one core, {wall:.1f} s (run while the GPU "
                         f"was measured)"}

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "float64" else "f32 stencils / f64 state", "data": "synthetic",
        "config": {"workload": w["name"] if args.precision == "float64" else w["name"].replace("plain float64", "mixed-precision"),
                   "precision": args.precision, "mesh_order": args.order, "cells": C_, "levels": L_, "scalars": S,
                   "state_bytes": state_bytes,
                   "l2": "inputs larger than L2 (device state %.1f GB)" % (state_bytes / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "cuda_graph": True, "bytes_per_cell_level_step": bytes_per_cell_level_step(S, True),
                   "autotune": tuning},
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches_per_step * K,
        "clocks": clocks.summary(), "stage_ms_per_step": stage_ms, "nonfinite": bad,
        "forms": forms,
    }
    return out


def run_reference(args, rank, world):
    """The reference's CPU float64 path on this workload (the numpy oracle port: the reference
    is Python and does not travel to the GPU machine).  A step is one large step of the same mesh
    and options from its prepared state; the K steps run as concurrent processes, one per
    host core, as many as the cores and the host memory allow in one round (the rest are
    not run, and the line says so).  Warm-up steps are not run: a CPU step keeps no warm
    state, and a level-6 step takes minutes."""
    w = WORKLOADS[args.workload]
    if rank != 0:
        return None
    procs = _oracle_procs(args.workload, args.steps)
    path, _ = _save_case(w)
    try:
        total, wall = cpu_throughput(w, procs=procs, nsteps=1, path=path)
    finally:
        os.unlink(path)
    value = total / wall
    sample = (f"{procs} of the {args.steps} requested large steps of the numpy oracle on this workload's own mesh "
              f"and options ({total // procs} cell-levels each), run concurrently as {procs} processes (one per "
              f"core, up to the cores and host memory available); wall {wall:.1f} s")
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * wall / procs, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["name"]}, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--workload", default="c1", choices=tuple(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-vjp", action="store_true",
                    help="only run two taped forward + reverse steps of the differentiation workload (for ncu)")
    ap.add_argument("--precision", default="float64", choices=("float64", "mixed"))
    ap.add_argument("--no-forms", action="store_true", help="skip the mixed and batched forms")
    ap.add_argument("--order", default="sfc", choices=("native", "sfc"),
                    help="mesh order on the device: generator order or Hilbert curve")
    ap.add_argument("--ensemble", type=int, default=96, help="members of the batched level-5 ensemble (0: skip)")
    ap.add_argument("--tile", default="auto", choices=("auto", "1", "2", "4"),
                    help="levels per thread of the u tendency: autotuned, or fixed (profiling)")
    ap.add_argument("--ensemble-groups", action="store_true",
                    help="also run the two-grid mixed ensemble (96 x 10242x41 + 32 x 40962x55, ~200 GB)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out))
        return
    if args.profile_vjp:
        import torch
        profile_dynamics_vjp(torch.device("cuda", 0))
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    out = run_gb300(args, rank, world)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
