#!/usr/bin/env python
"""Benchmark of the GB300 Repulsive-Surfaces hot path (one JSON line on stdout).

Workload (default ``--workload c2``): the Barnes-Hut tangent-point energy and its exact
differential on the 81,920-face icosphere of configuration c2 (level 6, spherical-harmonic
noise, alpha 6, beta 12, theta 0.25, leaf 8), FP32 pairs with Kahan accumulation, FP64 energy.
A step is one refit of the frozen tree to the (resident) positions plus one energy +
differential evaluation. The metric is the pair throughput in GFLOP/s, counting 61 FLOP per
pair interaction (one exact ordered pair or one lumped leaf-face/node term).

* ``value``: device-resident inputs, CUDA events on the library's stream around every step,
  L2 flushed (256 MiB write) between steps.
* ``e2e``: the same metric through the public C-ABI call with host buffers (positions in,
  energy and differential out) timed on the wall clock.
* ``roofline``: the pair kernel (bh_pair), FP32-bound, against the measured FP32 FMA peak.
* ``cpu_baseline``: the FP64 C++ restatement of the reference (the oracle; the Rust crate
  cannot be built here) on the host cores, one full evaluation of the same workload.
* ``--impl reference``: that CPU implementation as the reference arm.

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

FLOP_PER_INTERACTION = 61  # energy + gradient, SURVEY's count (FMA = 2, Kahan not counted)


def workload(name: str):
    from rs_gb300 import generators as gen

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


METRIC = "pair GFLOP/s, Barnes-Hut energy+differential (61 FLOP/interaction)"


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c3"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

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
    t_total = sum(ms) / 1e3
    if world > 1:
        tt = torch.tensor([t_total], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_total = float(tt.item())
    value = world * flop * args.steps / t_total / 1e9
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
    t_e2e = time.perf_counter() - t0
    if world > 1:
        tt = torch.tensor([t_e2e], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(tt.item())
    e2e = world * flop * args.steps / t_e2e / 1e9

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
                     "peak_source": "measured FP32 FMA throughput (rs_fp32_peak); "
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
