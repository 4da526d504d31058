#!/usr/bin/env python
"""Benchmark of the GB300 Repulsive-Surfaces hot path (one JSON line on stdout).

Default workload (``--workload flow``): Hs-flow steps on the 204,800-face torus of the step
configuration (320x320 grid, R = 1, r = 0.3, alpha 6, beta 12): Barnes-Hut energy and
differential (theta 0.25), hierarchical metric (chi 0.5, leaf 8), barycenter + area + volume
constraints (three right-hand sides per step), the fractional preconditioner, GMRES restart 30
to a true relative residual of 1e-6, Armijo line search and projection. One step = one
``rs_flow_step`` (trees, lists and solver rebuilt for the step, as the crate does). The noise
is N(0, 0.001) per coordinate: the specified N(0, 0.01) exceeds the torus' minor edge length
(0.0059) and crumples it so that no solver reaches 1e-6 (``--workload flow-spec`` runs it).

* ``value``: steps/s from CUDA events on the library's stream around every step (the steps
  move gigabytes, far above L2).
* ``e2e``: the same through the public call with the positions read back to the host after
  every step, on the wall clock; h2d/d2h bytes from the library's copy counters.
* ``roofline``: the dominant kernel of the step, the metric's near-field kernel (hm_rows):
  the bytes it must move per launch (the stored FP32 near weights and the channel values)
  against the measured HBM copy bandwidth, with its FP32 view (``compute``: counted FLOP
  against the measured FP32 FMA peak; the compensated arithmetic keeps it at the FP32 issue
  limit, far below HBM); the pair kernel is reported beside it.
* ``cpu_baseline`` / ``--impl reference``: complete FP64 steps of the C++ restatement of the
  reference (the oracle; the Rust crate cannot be built here) on the host cores, from the
  workload's start surface with the same settings: Barnes-Hut objective, hierarchical saddle
  solver with a sparse LDL^T of L' and the augmented preconditioner, three GMRES solves to
  1e-6, Armijo search and projection (about a minute on 16 host cores).

``--workload c2`` / ``c3``: the Barnes-Hut pair kernel alone (GFLOP/s, 61 FLOP per pair
interaction) on the 81,920-face icosphere or the specified torus.

Multi-GPU (torchrun): every rank runs an independent replica (the path has no exchange
step); value = all ranks' work / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "ddg-tools_gb300"))

FLOP_PER_INTERACTION = 61  # energy + gradient per interaction (FMA = 2; the compensation is not counted)


def replica_rate(units, seconds, world, device=None):
    """(rate, seconds) of `world` replicas that each processed `units` in their own `seconds`:
    all ranks' units over the slowest rank's time, from an all-reduce (max) of the times over
    the initialised process group (NCCL on the GPUs, gloo in the CPU tests)."""
    if world > 1:
        import torch
        import torch.distributed as dist

        tt = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        seconds = float(tt.item())
    return world * units / seconds, seconds


def workload(name: str):
    from rs_gb300 import generators as gen

    if name == "flow":
        P, F = gen.config_c3s()
        return P, F, 0.25, ("torus 320x320 R=1 r=0.3 (102,400 vertices, 204,800 faces), N(0,0.001) "
                            "noise per coordinate, seed 3")
    if name == "flow-spec":
        P, F = gen.config_c3()
        return P, F, 0.25, ("torus 320x320 R=1 r=0.3 (102,400 vertices, 204,800 faces), N(0,0.01) "
                            "noise per coordinate, seed 3 (as specified; crumpled)")
    if name == "matvec":
        P, F = gen.config_c3s()
        return P, F, 0.25, ("torus 320x320 R=1 r=0.3 (102,400 vertices, 204,800 faces), N(0,0.001) "
                            "noise per coordinate, seed 3")
    if name == "c2":
        P, F = gen.config_c2()
        return P, F, 0.25, ("icosphere level 6 (40,962 vertices, 81,920 faces), 8 spherical-"
                            "harmonic modes of degree <= 8, amplitude 0.05, seed 2")
    if name == "c3":
        P, F = gen.config_c3()
        return P, F, 0.25, "torus 320x320 R=1 r=0.3 (204,800 faces), N(0,0.01) noise, seed 3"
    raise SystemExit(f"unknown workload {name}")


class Clocks:
    """nvidia-smi samples (200 ms) while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def traffic_from_profiles(kernel: str, workload_name: str):
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    p = ROOT / "profiles" / f"{kernel}_{workload_name}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def _scaled_traffic(kernel, workload_name, units, units_profiled):
    """DRAM bytes per launch of a committed ncu summary, scaled by the units one launch
    processes here over the units of the profiled launch (the kernel's traffic grows with them)."""
    t = traffic_from_profiles(kernel, workload_name)
    return None if t is None else t * units / units_profiled


def cpu_baseline(P, F, theta, sizes, threads=None):
    """The FP64 oracle on the host cores: one evaluation of the same workload."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import rs_oracle as O

    O.build()
    n = threads or os.cpu_count() or 1
    O.set_threads(n)
    bh = O.BhTree(P, F, theta=theta)
    t0 = time.perf_counter()
    bh.energy_and_differential()
    dt = time.perf_counter() - t0
    n_int = sizes["pairs_exact"] + sizes["lumped_interactions"]
    return FLOP_PER_INTERACTION * n_int / dt / 1e9, dt, n


def run_reference(args, rank):
    if rank != 0:
        return 0
    P, F, theta, desc = workload(args.workload)
    sys.path.insert(0, str(ROOT / "oracle"))
    import rs_oracle as O

    O.build()
    n = os.cpu_count() or 1
    O.set_threads(n)
    bh = O.BhTree(P, F, theta=theta)
    n_int = bh.sizes()["pairs_exact"] + _lumped_interactions(bh)
    for _ in range(max(0, min(args.warmup, 1))):
        bh.energy_and_differential()
    times = []
    for _ in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        bh.energy_and_differential()
        times.append(time.perf_counter() - t0)
    dt = float(np.mean(times))
    v = FLOP_PER_INTERACTION * n_int / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "GFLOP/s", "n_gpus": args.gpus,
        "steps": len(times), "warmup": min(args.warmup, 1), "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": f"{args.workload}: {desc}", "theta": theta,
                                        "alpha": 6, "beta": 12, "leaf_size": 8},
        "cpu_baseline": {"value": v, "unit": "GFLOP/s", "cores": n, "kind": "port",
                         "sample": f"{len(times)} full evaluations of the workload, {n} threads; "
                                   "the reference crate (Rust) cannot be built here, so its C++ "
                                   "FP64 restatement runs"},
        "e2e": {"value": v, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _lumped_interactions(bh) -> int:
    t, L = bh.tree(), bh.lists()
    ns = (t["end"] - t["start"])[t["leaves"]].astype(np.int64)
    return int(np.sum(np.diff(L["lumped_off"]) * ns))


FLOW_METRIC = "Hs-flow steps/s @204,800 faces (plain preconditioner, rel.res 1e-6)"
# Near-field work of the metric per near entry and vector: w (m_p - m_q) added up, 3 FLOP per
# channel, C = 12 channels per vector (the near weights w are evaluated once per set-up, not per
# product; the compensated arithmetic executes about four times this count).
NEAR_FLOP_PER_ENTRY = 36
# Algorithmic bytes of one near-field launch (one vector, 12 channels): the stored FP32 weight
# pair of every near entry (8 B) and the channel values of every face as float pairs (96 B).
NEAR_BYTES_PER_ENTRY, NEAR_BYTES_PER_FACE = 8, 96


def hbm_peak():
    """The measured copy bandwidth of the GB300s (GB/s), else the stated fallback."""
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback (6.8 TB/s)"


def near_roofline(near_entries, n_faces, t_rows_ms, fp32_peak, traffic, kernel_ms):
    """The near-field kernel against HBM (the bytes it must move per launch), with its FP32
    view beside it (it executes the compensated difference form at the FP32 issue limit)."""
    algo = NEAR_BYTES_PER_ENTRY * near_entries + NEAR_BYTES_PER_FACE * n_faces
    peak, src = hbm_peak()
    gbs = algo / (t_rows_ms * 1e-3) / 1e9 if t_rows_ms else None
    tflops = NEAR_FLOP_PER_ENTRY * near_entries / (t_rows_ms * 1e-3) / 1e12 if t_rows_ms else None
    return {"bound": "hbm", "kernel": "hm_rows (metric near field, one vector)", "achieved": gbs, "peak": peak,
            "unit": "GB/s", "frac": (gbs / peak) if gbs else None, "peak_source": src,
            "work": f"{NEAR_BYTES_PER_ENTRY} B x {near_entries} near entries + {NEAR_BYTES_PER_FACE} B x "
                    f"{n_faces} faces per launch ({algo} B)",
            "traffic": traffic, "kernel_ms": kernel_ms,
            "compute": {"bound": "fp32", "achieved": tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                        "frac": (tflops / fp32_peak) if tflops else None,
                        "peak_source": "measured FP32 FMA throughput (rsp_fp32_peak, librsprobe.so)",
                        "work": f"{NEAR_FLOP_PER_ENTRY} FLOP x {near_entries} near entries per launch"}}
def flow_options(R):
    return R.flow_options(theta=0.25, hold_area=1, hold_volume=1, solver_chi=0.5, solver_restart=30,
                          solver_tolerance=1e-6, solver_max_iterations=300)


def cpu_flow_step(P, F, theta, threads=None, l0=0.0):
    """One complete FP64 step of the oracle on the host cores, with the GPU arm's settings: the
    Barnes-Hut objective (lists frozen for the step), the hierarchical saddle solver (metric tree
    chi 0.5, vertex fractional tree, sparse LDL^T of L', the augmented preconditioner), three
    GMRES solves (restart 30, true relative residual 1e-6), the Armijo search and the projection
    (Session::step_inner without remeshing and collision detection). Returns (steps/s, report,
    threads)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import rs_oracle as O

    O.build()
    n = threads or os.cpu_count() or 1
    O.set_threads(n)
    cons = O.Constraints().barycenter().area().volume()
    o = O.step_options(backend=1, energy_theta=theta, max_halvings=30, start_rule=3, start_value=2.0,
                       first_rule=1, first_value=1.0, l0=l0,
                       solver={"chi": 0.5, "restart": 30, "tolerance": 1e-6, "max_iterations": 300})
    t0 = time.perf_counter()
    rep = O.step(P, F, cons, o)
    dt = time.perf_counter() - t0
    return 1.0 / dt, rep, n


def _cpu_step_summary(rep, n, dt_label=""):
    return (f"one complete FP64 step of the workload's start surface (BH energy and differential, "
            f"solver build with a sparse LDL^T of L', 3 GMRES solves of {int(rep['gmres_iterations'])} "
            f"iterations in total, Armijo search, projection) by the C++ restatement of the reference "
            f"on {n} threads in {rep['s_total']:.1f} s{dt_label}: objective build {rep['s_objective']:.1f} s, "
            f"energy {rep['s_energy']:.1f} s, solver build {rep['s_solver_build']:.1f} s, solves "
            f"{rep['s_solve']:.1f} s, line search {rep['s_line_search']:.1f} s, projection "
            f"{rep['s_projection']:.1f} s; the reference crate (Rust) cannot be built here")


def run_reference_flow(args, rank):
    """The reference arm of the flow workloads: complete FP64 steps of the oracle, as many as
    fit in about two minutes after the first (at least one), from the workload's start surface."""
    if rank != 0:
        return 0
    P, F, theta, desc = workload(args.workload)
    t_all = time.perf_counter()
    v, rep, n = cpu_flow_step(P, F, theta)
    times = [1.0 / v]
    while time.perf_counter() - t_all + times[-1] < 120.0 and len(times) < args.steps:
        v2, _, _ = cpu_flow_step(P, F, theta)
        times.append(1.0 / v2)
    value = len(times) / sum(times)
    line = {
        "impl": "reference", "metric": FLOW_METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": len(times), "warmup": 0, "ms_per_step": 1e3 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": flow_config(args.workload, desc, theta, 1),
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": n, "kind": "port",
                         "sample": _cpu_step_summary(rep, n) + f"; {len(times)} step(s) timed, the same step "
                                   "from the same start each time (no warm-up: no JIT or cache to warm)"},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "step_report": {k: rep[k] for k in ("energy_before", "energy_after", "tau", "accepted", "gmres_iterations",
                                            "worst_residual", "newton_rounds")},
    }
    print(json.dumps(line), flush=True)
    return 0


def flow_config(workload_name, desc, theta, world):
    return {"workload": f"{workload_name}: {desc}", "theta": theta, "chi": 0.5, "alpha": 6, "beta": 12,
            "leaf_size": 8, "constraints": "barycenter + area + volume (3 right-hand sides per step)",
            "gmres": "restart 30, true relative residual 1e-6, at most 300 iterations",
            "line_search": "Armijo c 1e-2, start: farthest vertex one mean edge, then twice the last tau",
            "l2": "not flushed: every step moves several GB (trees, lists, solver rebuilt)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def bench_flow(args, rank, world, local):
    import torch

    import rs_gb300 as R

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    warmup = max(3, args.warmup)
    P, F, theta, desc = workload(args.workload)
    ctx = R.Context(local)
    dev = torch.device(f"cuda:{local}")
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    flow = R.Flow(F, P, flow_options(R), ctx)
    t0 = time.perf_counter()
    first = flow.step()  # the first step from the start surface (the CPU arm's step)
    first_wall = time.perf_counter() - t0
    for _ in range(warmup - 1):
        flow.step()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    reps = []
    if world > 1:
        torch.distributed.barrier()
    Q0 = flow.positions()  # the start of the timed steps, for the e2e run over the same steps
    torch.cuda.synchronize(dev)
    l0 = ctx.launch_count()
    with Clocks(local) as clk:
        for a, b in evs:
            a.record(stream)
            reps.append(flow.step())
            b.record(stream)
        stream.synchronize()
    launches = ctx.launch_count() - l0
    ms = [a.elapsed_time(b) for a, b in evs]
    value, t_total = replica_rate(args.steps, sum(ms) / 1e3, world, dev)

    # e2e: the public call with host positions read back after every step, wall clock, over the
    # same steps: a flow created from the positions where the timed steps started
    if world > 1:
        torch.distributed.barrier()
    flow_e = R.Flow(F, Q0, flow_options(R), ctx)
    c0 = R.copy_counters()
    t0 = time.perf_counter()
    e2e_reps = []
    for _ in range(args.steps):
        e2e_reps.append(flow_e.step())
        Q = flow_e.positions()
    c1 = R.copy_counters()
    e2e, t_e2e = replica_rate(args.steps, time.perf_counter() - t0, world, dev)

    # the learned preconditioner on the same flow (continuing from here), plain as its fallback
    learned = None
    try:
        from rs_gb300 import learned as LR

        lm = R.LearnedModel(seed=1, ctx=ctx)
        if LR.load(lm):
            flow.set_learned(lm, cheap_steps=2, max_iterations=100)
            lreps, t0 = [], time.perf_counter()
            for _ in range(max(1, min(3, args.steps))):
                lreps.append(flow.step())
            t_l = time.perf_counter() - t0
            flow.set_learned(None)
            learned = {"steps_per_s": len(lreps) / t_l, "vs_plain_e2e": (len(lreps) / t_l) / (args.steps / t_e2e),
                       "steps": len(lreps), "learned_solves": int(sum(r["learned_solves"] for r in lreps)),
                       "fallbacks_to_plain": int(sum(r["learned_fallbacks"] for r in lreps)),
                       "relative_residual_max": max(r["relative_residual"] for r in lreps),
                       "setting": "y = plain preconditioner with 2 CG steps, z = y + network correction; "
                                  "GMRES capped at 100 iterations before the plain fallback"}
    except R.RsError as e:
        learned = {"error": str(e)}
    # the step configuration's own noise, N(0, 0.01) (1.7 minor edge lengths: a crumpled torus):
    # one step from it with the same settings, the residual GMRES reaches there, and the
    # operator's linearity defect |A(x (1 + 2^-20)) / (1 + 2^-20) - A x| / |A x| on the
    # direction's solution, which shows that conditioning, not rounding, limits the solve
    # the step configuration's own noise, N(0, 0.01) (1.7 minor edge lengths: a crumpled torus):
    # one step from it with the headline settings, the lowest residual each of the step's three
    # solves reaches, and the operator's linearity defect |A(x (1 + 2^-20)) / (1 + 2^-20) - A x|
    # / |A x|, which shows that conditioning, not rounding, limits the solves
    flow_spec = None
    if args.workload == "flow":
        Ps, Fs = workload("flow-spec")[:2]
        flow_spec = {"noise": 0.01}
        try:
            rs = R.Flow(Fs, Ps, flow_options(R), ctx).step()
            flow_spec["step"] = {"relative_residual": rs["relative_residual"], "accepted": rs["accepted"]}
        except R.RsError as e:
            flow_spec["step"] = {"error": str(e)}
        try:
            bs = R.BhTree.build(Fs, Ps, R.BhOptions(0.25, 8), ctx)
            Es, dEs = bs.energy_and_differential(R.Exponents())
            from rs_gb300 import learned as LR

            ga, gv = LR._constraint_gradients(Ps, Fs)
            out = {}
            for clamp in (0, 1):  # 1: the multigrid on the Laplacian without its negative weights
                Ss = R.SaddleSolver(Fs, Ps, R.Exponents(), R.solver_options(
                    chi=0.5, restart=30, tolerance=1e-6, max_iterations=300, clamp_laplacian=clamp), ctx)
                rhs = np.zeros((3, Ss.n))
                rhs[0, :Ss.n_dofs], rhs[1, :Ss.n_dofs], rhs[2, :Ss.n_dofs] = ga.ravel(), gv.ravel(), dEs.ravel()
                try:
                    Ss.solve_many(rhs)
                except R.RsError:
                    pass
                best = []
                for q in range(3):
                    cyc = Ss.history(q)[1]
                    best.append(float(min(cyc)) if len(cyc) else None)
                v = np.zeros((1, Ss.n))
                v[0, :Ss.n_dofs] = dEs.ravel() / np.linalg.norm(dEs)
                a1 = Ss.apply(v)[0]
                a2 = Ss.apply(v * (1.0 + 2.0 ** -20))[0] / (1.0 + 2.0 ** -20)
                out["clamped" if clamp else "cotan"] = {
                    "lowest_cycle_residual": best,
                    "operator_linearity_defect": float(np.linalg.norm(a2 - a1) / np.linalg.norm(a1))}
                del Ss
            flow_spec.update(energy=float(Es), solves=out,
                             note="the specified N(0, 0.01) torus with the headline settings: the lowest "
                                  "residual of the three solves (area, volume, direction rows) in 300 "
                                  "iterations, and the operator's linearity defect")
        except R.RsError as e:
            flow_spec["error"] = str(e)
    # one step with the collision cap of the line search (rs_flow_options.ccd, the crate's
    # default line search) on the current surface: its cost inside a step
    with_ccd = None
    try:
        o = flow_options(R)
        o.ccd = 1
        fc = R.Flow(F, Q, o, ctx)
        rc = fc.step()
        with_ccd = {"seconds_step": rc["seconds"], "seconds_ccd": rc["seconds_ccd"],
                    "tau_ccd": rc["tau_ccd"], "tau0": rc["tau0"], "accepted": rc["accepted"],
                    "note": "one step after the timed region; band of the start, then first contact "
                            "of x - t d on [0, tau0]"}
        del fc
    except R.RsError as e:
        with_ccd = {"error": str(e)}
    # phases of one step's solve (three right-hand sides) on the current surface
    solve_phases = None
    try:
        S = R.SaddleSolver(F, Q, R.Exponents(), R.solver_options(chi=0.5, restart=30, tolerance=1e-6,
                                                                  max_iterations=300), ctx)
        bh0 = R.BhTree.build(F, Q, R.BhOptions(theta, 8), ctx)
        _, dE = bh0.energy_and_differential(R.Exponents())
        from rs_gb300 import learned as LR

        ga, gv = LR._constraint_gradients(Q, F)
        rhs = np.zeros((3, S.n))
        rhs[0, :S.n_dofs], rhs[1, :S.n_dofs], rhs[2, :S.n_dofs] = ga.ravel(), gv.ravel(), dE.ravel()
        solve_phases = {k: round(v, 2) for k, v in S.profile(rhs).items()}
        solve_phases["iterations"] = [len(S.history(q)[0]) for q in range(3)]
        solve_phases["multigrid_levels"] = S.multigrid_levels()
        solve_phases["build_s"] = {k: round(v, 4) for k, v in S.build_times().items()}
        del S, bh0
    except R.RsError as e:
        solve_phases = {"error": str(e)}
    # roofline: the metric's near-field kernel on the current surface (one vector per launch)
    m = R.FaceMetricTree(F, Q, R.Exponents(), R.ClusterTreeOptions(chi=0.5), ctx)
    mst = m.stats()
    mprof = m.profile(1, 5)
    t_rows = mprof.get("metric_rows")
    peak = ctx.fp32_peak_tflops()
    # the pair kernel on the same surface
    bh = R.BhTree.build(F, Q, R.BhOptions(theta, 8), ctx)
    bs = bh.sizes()
    n_int = bs["pairs_exact"] + bs["lumped_interactions"]
    bprof = bh.profile(R.Exponents(), reps=5)
    t_pair = bprof.get("bh_pair_grad")
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        if rank != 0:
            dist.destroy_process_group()
            return 0

    def mean(key, rr=reps):
        return float(np.mean([r[key] for r in rr]))

    its = [r["gmres_area"] + r["gmres_volume"] + r["gmres_direction"] for r in reps]
    line = {
        "metric": FLOW_METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded mesh generator of the configuration)",
        "config": flow_config(args.workload, desc, theta, world),
        "implementation": {"gmres": "FP64 Arnoldi (CGS2) on the device",
                           "preconditioner": "fractional (plain); L' by 6 multigrid-preconditioned CG steps"},
        "steps_report": {
            "gmres_iterations_per_step": float(np.mean(its)),
            "gmres_iterations": [[int(r["gmres_area"]), int(r["gmres_volume"]), int(r["gmres_direction"])]
                                 for r in reps],
            "relative_residual_max": max(r["relative_residual"] for r in reps),
            "energy": [reps[0]["energy_before"], reps[-1]["energy_after"]],
            "accepted": int(sum(r["accepted"] for r in reps)),
            "seconds": {k: mean(k) for k in ("seconds", "seconds_tree", "seconds_energy", "seconds_solver_build",
                                               "seconds_solve", "seconds_line_search", "seconds_projection")},
        },
        "e2e": {"value": e2e, "unit": "steps/s",
                "h2d_bytes_per_step": int((c1[0] - c0[0]) / args.steps),
                "d2h_bytes_per_step": int((c1[1] - c0[1]) / args.steps)},
        "roofline": near_roofline(mst["near_entries"], len(F), t_rows, peak,
                                  _scaled_traffic("hm_rows", "matvec", mst["near_entries"], 103578780), mprof),
        "pair_kernel": {"gflops": FLOP_PER_INTERACTION * n_int / (t_pair * 1e-3) / 1e9 if t_pair else None,
                        "interactions": n_int, "ms": t_pair,
                        "frac": (FLOP_PER_INTERACTION * n_int / (t_pair * 1e-3) / 1e12 / peak) if t_pair else None},
        "first_step": {"wall_s": first_wall, "gmres_iterations": int(first["gmres_area"] + first["gmres_volume"]
                                                                   + first["gmres_direction"]),
                       "energy": [first["energy_before"], first["energy_after"]],
                       "note": "the first (warm-up) step from the start surface, the step the CPU arm "
                               "times; host wall clock including the library's first-use set-up"},
        "solve_phases_ms": solve_phases,
        "flow_spec": flow_spec,
        "learned_preconditioner": learned,
        "step_with_ccd": with_ccd,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, crep, n = cpu_flow_step(P, F, theta)
        line["cpu_baseline"] = {"value": v, "unit": "steps/s", "cores": n, "kind": "port",
                                "sample": _cpu_step_summary(crep, n)}
    if world > 1:
        torch.distributed.destroy_process_group()
    print(json.dumps(line), flush=True)
    return 0


MATVEC_METRIC = "Hs metric products/s @204,800 faces (hierarchical, chi 0.5, one vector)"


def bench_matvec(args, rank, world, local):
    """The hierarchical metric product alone (rs_metric_apply_device, one vector per step)."""
    import torch

    import rs_gb300 as R

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    warmup = max(3, args.warmup)
    P, F, theta, desc = workload(args.workload)
    ctx = R.Context(local)
    dev = torch.device(f"cuda:{local}")
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    m = R.FaceMetricTree(F, P, R.Exponents(), R.ClusterTreeOptions(chi=0.5), ctx)
    st = m.stats()
    with torch.cuda.stream(stream):
        x = torch.from_numpy(np.random.default_rng(0).standard_normal(3 * len(P))).to(dev)
        y = torch.zeros_like(x)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
        for _ in range(warmup):
            m.apply_device(x.data_ptr(), y.data_ptr(), 1)
        stream.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        l0 = ctx.launch_count()
        with Clocks(local) as clk:
            for a, b in evs:
                flush.fill_(1)
                a.record(stream)
                m.apply_device(x.data_ptr(), y.data_ptr(), 1)
                b.record(stream)
            stream.synchronize()
        launches = ctx.launch_count() - l0
    value, t_total = replica_rate(args.steps, sum(a.elapsed_time(b) for a, b in evs) / 1e3, world, dev)
    xh = np.random.default_rng(1).standard_normal(3 * len(P))
    m.apply(xh)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        yh = m.apply(xh)
    e2e, _ = replica_rate(args.steps, time.perf_counter() - t0, world, dev)
    prof = m.profile(1, 5)
    peak = ctx.fp32_peak_tflops()
    t_rows = prof.get("metric_rows")
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        if rank != 0:
            dist.destroy_process_group()
            return 0
    line = {
        "metric": MATVEC_METRIC, "value": value, "unit": "products/s", "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded mesh generator of the configuration)",
        "config": {"workload": f"matvec: {desc}", "chi": 0.5, "alpha": 6, "beta": 12, "leaf_size": 8,
                   "leaf_pairs": 64, **st, "l2": "flushed (256 MiB) between steps",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": "products/s",
                "h2d_bytes_per_step": int(xh.nbytes), "d2h_bytes_per_step": int(xh.nbytes)},
        "roofline": near_roofline(st["near_entries"], len(F), t_rows, peak, traffic_from_profiles("hm_rows", "matvec"),
                                  prof),
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import rs_oracle as O

        O.build()
        n = os.cpu_count() or 1
        O.set_threads(n)
        om = O.FaceMetricTree(P, F, chi=0.5)
        t0 = time.perf_counter()
        om.apply(xh)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "products/s", "cores": n, "kind": "port",
                                "sample": f"one product ({dt:.2f} s) by the FP64 C++ restatement, {n} threads"}
    if world > 1:
        torch.distributed.destroy_process_group()
    print(json.dumps(line), flush=True)
    return 0


def ccd_motion(P, F, reach=2.0, seed=5):
    """A smooth seeded velocity field on the surface, scaled so that the fastest vertex moves
    `reach` mean edge lengths by t = 1 (a line-search trial of the flow moves it one to two)."""
    rng = np.random.default_rng(seed)
    k = rng.normal(size=(4, 3))
    ph = rng.uniform(0, 2 * np.pi, (4, 3))
    vel = sum(np.sin(P @ k[i][:, None] * 2.0 + ph[i]) for i in range(4))
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]).astype(np.int64)
    e = np.unique(np.sort(e, axis=1), axis=0)
    mel = np.linalg.norm(P[e[:, 0]] - P[e[:, 1]], axis=1).mean()
    return np.ascontiguousarray(vel * (reach * mel / np.linalg.norm(vel, axis=1).max()))


def bench_ccd(args, rank, world, local):
    """Continuous collision detection of the 204,800-face torus against itself along a smooth
    motion (rs_ccd_first_contact: host arrays in, tau_max out; one call per step)."""
    import torch

    import rs_gb300 as R

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    warmup = max(3, args.warmup)
    P, F, _, desc = workload("flow")
    V = ccd_motion(P, F)
    ctx = R.Context(local)
    c = R.CcdSurface(F, len(P), ctx)
    for _ in range(warmup):
        r = c.first_contact(P, V, 1.0)
    if world > 1:
        torch.distributed.barrier()
    l0 = ctx.launch_count()
    ms = []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            r = c.first_contact(P, V, 1.0)
            ms.append((time.perf_counter() - t0) * 1e3)
    launches = ctx.launch_count() - l0
    value, t_total = replica_rate(args.steps, sum(ms) / 1e3, world, torch.device(f"cuda:{local}"))
    if world > 1:
        torch.distributed.barrier()
        if rank != 0:
            torch.distributed.destroy_process_group()
            return 0
    line = {
        "metric": "CCD first_contact calls/s @204,800 faces (self contacts, gap 0.05 of the mean edge)",
        "value": value, "unit": "calls/s", "n_gpus": world, "steps": args.steps, "warmup": warmup,
        "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh generator and motion)",
        "config": {"workload": f"ccd: {desc}; smooth seeded velocity, fastest vertex 2 mean edges by t = 1",
                   "tau_end": 1.0, **{k: r[k] for k in ("tau_max", "contact", "windows", "pairs_tested",
                                                      "close_pairs", "touching_pairs", "evaluations")},
                   "l2": "inputs uploaded from the host in every call",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": value, "unit": "calls/s", "h2d_bytes_per_step": int(P.nbytes + V.nbytes),
                "d2h_bytes_per_step": 64 * int(r["windows"])},
        "pairs_per_s": r["pairs_tested"] * value, "evaluations_per_s": r["evaluations"] * value,
        "roofline": None,
        "roofline_note": ("the narrow phase (64 % of the GPU time) is bound by the FP64 pipe, ~70 % active "
                          "where it runs (ncu, profiles/ccd_first_contact.md); no FP64 peak is measured "
                          "on this pool, so no fraction is reported"),
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = ccd_cpu(P, F, V)
    if world > 1:
        torch.distributed.destroy_process_group()
    print(json.dumps(line), flush=True)
    return 0


def ccd_cpu(P, F, V, calls=1):
    """The oracle's first_contact of the same motion on all host cores (x-sweep broad phase)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import rs_oracle as O

    O.build()
    n = os.cpu_count() or 1
    O.set_threads(n)
    t0 = time.perf_counter()
    for _ in range(calls):
        r = O.ccd_first_contact(F, P, V, 1.0)
    dt = (time.perf_counter() - t0) / calls
    return {"value": 1.0 / dt, "unit": "calls/s", "cores": n, "kind": "port", "tau_max": r["tau_max"],
            "sample": f"{calls} call(s) of the FP64 C++ restatement on {n} threads ({dt:.2f} s each)"}


METRIC = "pair GFLOP/s, Barnes-Hut energy+differential (61 FLOP/interaction)"


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="flow", choices=["flow", "flow-spec", "matvec", "c2", "c3", "ccd"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 5 if args.workload.startswith("flow") else 20
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if args.workload == "ccd":
            if rank == 0:
                P, F, _, desc = workload("flow")
                V = ccd_motion(P, F)
                cb = ccd_cpu(P, F, V, calls=max(1, min(args.steps, 3)))
                print(json.dumps({
                    "impl": "reference", "metric": "CCD first_contact calls/s @204,800 faces (self contacts, gap "
                    "0.05 of the mean edge)", "value": cb["value"], "unit": "calls/s", "n_gpus": 1,
                    "steps": max(1, min(args.steps, 3)), "warmup": 0, "ms_per_step": 1e3 / cb["value"],
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                    "data": "synthetic (seeded mesh generator and motion)",
                    "config": {"workload": f"ccd: {desc}; smooth seeded velocity, fastest vertex 2 mean edges by t = 1",
                               "tau_end": 1.0},
                    "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "calls/s", "h2d_bytes_per_step": 0,
                                                "d2h_bytes_per_step": 0}}), flush=True)
            return 0
        if args.workload.startswith("flow"):
            return run_reference_flow(args, rank)
        return run_reference(args, rank)
    if args.workload.startswith("flow"):
        return bench_flow(args, rank, world, local)
    if args.workload == "matvec":
        return bench_matvec(args, rank, world, local)
    if args.workload == "ccd":
        return bench_ccd(args, rank, world, local)

    import torch

    import rs_gb300 as R

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    warmup = max(3, args.warmup)
    P, F, theta, desc = workload(args.workload)
    ctx = R.Context(local)
    ex = R.Exponents(6.0, 12.0)
    tree = R.BhTree.build(F, P, R.BhOptions(theta, 8), ctx)
    s = tree.sizes()
    n_int = s["pairs_exact"] + s["lumped_interactions"]
    flop = FLOP_PER_INTERACTION * n_int
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{local}")
    dev = torch.device(f"cuda:{local}")
    with torch.cuda.stream(stream):
        pos = torch.from_numpy(P.copy()).to(dev)
        e_dev = torch.zeros(1, dtype=torch.float64, device=dev)
        d_dev = torch.zeros(P.shape, dtype=torch.float64, device=dev)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step():
        tree.refit_device(pos.data_ptr())
        tree.energy_and_differential_device(ex, e_dev.data_ptr(), d_dev.data_ptr())

    with torch.cuda.stream(stream):
        for _ in range(warmup):
            step()
        stream.synchronize()
        # ---- value: device-resident, events around every step, L2 flushed between steps
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        l0 = ctx.launch_count()
        with Clocks(local) as clk:
            for a, b in evs:
                flush.fill_(1)
                a.record(stream)
                step()
                b.record(stream)
            stream.synchronize()
        launches = ctx.launch_count() - l0
        torch.cuda.synchronize(dev)
    ms = [a.elapsed_time(b) for a, b in evs]
    value, t_total = replica_rate(flop * args.steps / 1e9, sum(ms) / 1e3, world, dev)
    energy = float(e_dev.item())

    # ---- e2e: public C-ABI entry points with host buffers
    if world > 1:
        torch.distributed.barrier()
    tree.refit(P)
    tree.energy_and_differential(ex)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tree.refit(P)
        E2, dE2 = tree.energy_and_differential(ex)
    e2e, _ = replica_rate(flop * args.steps / 1e9, time.perf_counter() - t0, world, dev)

    # ---- roofline of the pair kernel (events around each launch on the library stream)
    prof = tree.profile(ex, reps=max(3, min(args.steps, 10)))
    t_pair = prof.get("bh_pair_grad")
    peak = ctx.fp32_peak_tflops()
    achieved = flop / (t_pair * 1e-3) / 1e12 if t_pair else None
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        if rank != 0:
            dist.destroy_process_group()
            return 0
    line = {
        "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded mesh generators of the configuration)",
        "config": {"workload": f"{args.workload}: {desc}", "theta": theta, "alpha": 6, "beta": 12,
                   "leaf_size": 8, "interactions": n_int, "pairs_exact": s["pairs_exact"],
                   "lumped_interactions": s["lumped_interactions"], "l2": "flushed (256 MiB) between steps",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "evals_per_s": world * args.steps / t_total,
        "energy": energy,
        "e2e": {"value": e2e, "unit": "GFLOP/s", "h2d_bytes_per_step": int(P.nbytes),
                "d2h_bytes_per_step": int(P.nbytes + 8)},
        "roofline": {"bound": "fp32", "kernel": "bh_pair_grad", "achieved": achieved,
                     "peak": peak, "unit": "TFLOP/s",
                     "frac": (achieved / peak) if achieved else None,
                     "peak_source": "measured FP32 FMA throughput (rsp_fp32_peak, librsprobe.so); "
                                    "MEASURED_PEAKS.json has no FP32 figure",
                     "traffic": traffic_from_profiles("bh_pair", args.workload),
                     "kernel_ms": prof},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, dt, n = cpu_baseline(P, F, theta, s)
        line["cpu_baseline"] = {"value": v, "unit": "GFLOP/s", "cores": n, "kind": "port",
                                "sample": f"one full evaluation of the workload ({dt:.2f} s) by the "
                                          f"FP64 C++ restatement, {n} threads"}
    if world > 1:
        torch.distributed.destroy_process_group()
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
