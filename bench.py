#!/usr/bin/env python
"""Benchmark: converged eigenpairs/s of the cyclic-symmetry modal solve on GB300.

Workload: the batched rpm sweep on the rotating bladed-disk sector (config-1 mesh:
40x24x6 hub + 30x10x2 twisted blade, 57,897 nodes, titanium, 36 sectors), 24 speeds in
linspace(0, 15000) rpm x harmonic indices 0..18, num_modes = 10, rotating effects (spin
softening + stress stiffening), standard Hermitian shift-invert path.  A step is one speed
of the sweep (all 19 harmonic problems: assembly, prestress, projections, factorisations,
Lanczos, expansion).  Speeds are taken in order, rank r of N takes speeds r, r+N, ...
(weak scaling: per-GPU work fixed).

value   eigenpairs/s of the mixed path (FP32 LDL^H + FP64 refinement), counting returned
        eigenpairs that converged and lie within 1e-6 relative frequency error of the plain
        FP64 GPU path on the same problem (verified after the timed region), over the device
        time (CUDA events on the library's stream) of the timed steps.
e2e     the same count over the wall-clock of the public API call (solve_at_rpm through the
        C ABI, speed and harmonic list in, frequencies + mode shapes copied back to host).
Inputs are larger than L2 (fronts of tens of GB), so no L2 flush is needed.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RPMS = np.linspace(0.0, 15000.0, 24)
METRIC = "converged eigenpairs/s @1e-6 rel freq err (mixed FP32 LDL^H + FP64 refinement, 1 GB300)"
UNIT = "eigenpairs/s"
WORKLOAD = "config-1 bladed-disk sector rpm sweep (57,897 nodes, 24 speeds x 19 harmonics, 10 modes)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--harmonics", default="all", help="comma list or 'all'")
    ap.add_argument("--num-modes", type=int, default=10)
    ap.add_argument("--no-verify", action="store_true", help="skip the FP64 verification pass")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the served request-stream sample")
    ap.add_argument("--serve-requests", type=int, default=12)
    ap.add_argument("--serve-max-nodes", type=int, default=30000,
                    help="largest sector of the request-stream sample (the full stream goes to 200000)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def shard_speeds(rpms, rank: int, world: int):
    """Speeds of this rank: r, r + N, r + 2N, ... (replicas only; no data-path collective)."""
    return list(rpms[rank::world])


def harmonics_arg(a):
    return [] if a == "all" else [int(x) for x in a.split(",")]


def count_distinct_verified(mixed, fp64, tol=1e-6):
    """Verified eigenpairs counting each degenerate (x, conj x) pair once.  On the standard path a
    harmonic 0 < k < N/2 returns every eigenpair twice, at positions 2q and 2q+1 with the same
    frequency (src/cyclic_solver.cpp:1162-1183); standing harmonics (whirl 0) return distinct
    ones."""
    ref = {r.harmonic_index: np.asarray(r.frequencies) for r in fp64}
    n = 0
    for r in mixed:
        f = np.asarray(r.frequencies)
        g = ref.get(r.harmonic_index)
        if g is None or len(g) != len(f) or not r.converged:
            continue
        ok = np.abs(f - g) <= tol * np.maximum(np.abs(g), 1e-300)
        paired = len(f) > 0 and bool(np.all(np.asarray(r.whirl_direction) != 0))
        n += int(np.sum(ok[0::2])) if paired else int(np.sum(ok))
    return n


def count_verified(mixed, fp64, tol=1e-6):
    ref = {r.harmonic_index: np.asarray(r.frequencies) for r in fp64}
    n_ok = n_all = 0
    worst = 0.0
    for r in mixed:
        f = np.asarray(r.frequencies)
        n_all += len(f)
        g = ref.get(r.harmonic_index)
        if g is None or len(g) != len(f) or not r.converged:
            continue
        err = np.abs(f - g) / np.maximum(np.abs(g), 1e-300)
        worst = max(worst, float(err.max()) if len(err) else 0.0)
        n_ok += int(np.sum(err <= tol))
    return n_ok, n_all, worst


def cpu_baseline_sample(rpm: float, F_target: float, threads: int = 1, all_harmonics: bool = False):
    """Oracle (CPU restatement of the reference path) on a bounded sample: harmonic k=1 (or
    every harmonic, over `threads` host threads as the reference's thread pool does) of a
    config-1-family sector small enough for ~10-60 s of CPU work, full pipeline (assembly,
    prestress, projections, simplicial LDL^H, Lanczos).  The eigenpairs/s is scaled to the
    config-1 problem by the ratio of factorisation flops (the dominant CPU cost)."""
    from oracle import orc
    from turbomodal_gb300.meshgen import TITANIUM, sector_mesh
    import scipy.sparse as sp

    if all_harmonics:   # all 19 harmonics: a smaller sector keeps a step to ~30 s of host time
        m = sector_mesh(14, 8, 3, num_sectors=36, jitter=0.02, seed=11,
                        blade=dict(ns=9, nc=4, nb=2, span=0.12, chord=0.05, thick=0.004, twist_deg=30.0))
    else:
        m = sector_mesh(18, 10, 4, num_sectors=36, jitter=0.02, seed=11,
                        blade=dict(ns=12, nc=5, nb=2, span=0.12, chord=0.05, thick=0.004, twist_deg=30.0))
    om = orc.OracleModel(m, TITANIUM)
    t0 = time.perf_counter()
    om.prepare(rpm)
    ks = list(range(m.num_sectors // 2 + 1)) if all_harmonics else [1]
    res = om.solve(rpm, 10, harmonic_indices=ks, max_threads=threads, with_shapes=True)
    t = time.perf_counter() - t0
    n_pairs = sum(len(r["frequencies"]) for r in res)
    Kk, Mk = om.matrix("Kk", k=1), om.matrix("Mk", k=1)
    P = sp.tril(sp.csc_matrix((abs(Kk) + abs(Mk)) > 0, dtype=float)).tocsc()
    _, _, cc = orc.ldl_symbolic(P)
    F_sample = 4.0 * float(np.sum(cc.astype(np.float64) ** 2))
    t_scaled = t * F_target / F_sample
    which = f"harmonics 0..{m.num_sectors // 2} on {threads} threads" if all_harmonics else "harmonic k=1 on 1 thread"
    return {"value": n_pairs / t_scaled, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"oracle, {which} at {rpm:.0f} rpm of a {m.num_nodes()}-node config-1-family sector "
                       f"({t:.1f} s, {n_pairs} eigenpairs), time scaled by factorisation flops "
                       f"{F_target:.3g}/{F_sample:.3g} to the config-1 problem"),
            "sample_seconds": t}


def run_reference(args, ws, rank, pg):
    """Reference arm: the reference's CPU algorithm (the oracle restatement; the reference itself
    needs Eigen and Spectra, which are not available) on the same workload family."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    # factorisation flops of the config-1 harmonic operator (host symbolic analysis only)
    F_target = 3.79696e12
    vals = []
    for _ in range(args.warmup + args.steps):
        vals.append(cpu_baseline_sample(RPMS[1], F_target, threads=cores, all_harmonics=True))
    v = float(np.mean([x["value"] for x in vals[args.warmup:]]))
    ms = float(np.mean([x["sample_seconds"] for x in vals[args.warmup:]])) * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": vals[-1]["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank, pg)
        return
    import torch

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    from turbomodal_gb300 import build as tmg_build
    from turbomodal_gb300.meshgen import TITANIUM, config_mesh
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    tmg_build.build()
    mesh = config_mesh(1)
    hi = harmonics_arg(args.harmonics)
    my_rpms = shard_speeds(RPMS, rank, ws)
    solver = CyclicSymmetrySolver(mesh, TITANIUM, device=local, precision="mixed")
    order = list(my_rpms) * (1 + (args.warmup + args.steps) // max(1, len(my_rpms)))
    warm, timed = order[: args.warmup], order[args.warmup: args.warmup + args.steps]
    for rpm in warm:
        solver.solve_at_rpm(rpm, args.num_modes, hi, precision="mixed")
    torch.cuda.synchronize()
    barrier(pg)
    clocks = ClockSampler(local)
    clocks.start()
    dev_ms, wall_s, results, launches, d2h = [], [], [], 0, 0
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    for rpm in timed:
        t0 = time.perf_counter()
        res = solver.solve_at_rpm(rpm, args.num_modes, hi, precision="mixed")
        wall_s.append(time.perf_counter() - t0)
        tm = solver.last_timing()
        dev_ms.append(tm["device_ms"])
        launches += int(tm["kernel_launches"])
        d2h += sum(r.frequencies.nbytes + r.mode_shapes.nbytes + r.whirl_direction.nbytes for r in res)
        results.append(res)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    barrier(pg)
    # verification against the plain FP64 GPU path (untimed) and its own throughput
    n_ok = n_all = 0
    n_distinct = None
    worst = 0.0
    fp64_ms = 0.0
    fp64_pairs = 0
    if not args.no_verify:
        n_distinct = 0
        for rpm, res in zip(timed, results):
            ref = solver.solve_at_rpm(rpm, args.num_modes, hi, precision="fp64")
            fp64_ms += solver.last_timing()["device_ms"]
            fp64_pairs += sum(len(r.frequencies) for r in ref if r.converged)
            a, b, w = count_verified(res, ref)
            n_ok += a
            n_all += b
            n_distinct += count_distinct_verified(res, ref)
            worst = max(worst, w)
    else:
        n_ok = n_all = sum(len(r.frequencies) for res in results for r in res)
    # roofline of the dominant kernel: the shift-invert triangular-solve graph of the batch of
    # complex harmonics (HBM bound), timed live with CUDA events in one extra profiled solve
    mesh_k = [k for k in (hi or range(mesh.num_sectors // 2 + 1)) if 0 < k < mesh.num_sectors / 2]
    solver.set_profiling(True)
    solver.solve_at_rpm(timed[0], args.num_modes, mesh_k, precision="mixed")
    prof = solver.profile_solve()
    solver.set_profiling(False)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    per_launch_bytes = prof["bytes"] / max(prof["count"], 1)
    per_launch_s = prof["ms"] / max(prof["count"], 1) / 1e3
    achieved = per_launch_bytes / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    traffic = None   # DRAM bytes of one batched solve from an ncu capture of this workload
    tr_path = os.path.join(ROOT, "profiles", "trisolve_cfg1_traffic.txt")
    if os.path.exists(tr_path):
        with open(tr_path) as fh:
            for line in fh:
                if line.startswith("dram_bytes_per_solve"):
                    traffic = float(line.split("=")[1])
    t_dev = max_over_ranks(pg, sum(dev_ms) / 1e3)
    t_wall = max_over_ranks(pg, sum(wall_s))
    tot_ok = sum_over_ranks(pg, n_ok)
    tot_all = sum_over_ranks(pg, n_all)
    tot_distinct = sum_over_ranks(pg, n_distinct or 0)
    serving = None
    if rank == 0 and not args.no_serve:
        # served request stream (Poisson arrivals, mixed sizes, admission by memory budget)
        from turbomodal_gb300.serve import ModalServer, latency_summary, request_stream

        reqs = request_stream(args.serve_requests, seed=2024, rate_hz=20.0, min_nodes=2000,
                              max_nodes=args.serve_max_nodes)
        srv = ModalServer(device=local, budget_bytes=150 << 30, max_inflight=4)
        done = srv.serve(reqs)
        srv.close()
        serving = latency_summary(done)
        serving["sample"] = (f"{len(reqs)} requests, Poisson 20 req/s, config-0/1-style sectors of 2000-"
                             f"{args.serve_max_nodes} nodes (log-uniform), 24/36/48 sectors, rpm U(0,15000), "
                             "5-20 modes, 1-19 random harmonics, mixed precision, 150 GB budget, 4 in flight")
    if rank == 0:
        cpu = None
        if ws == 1 and not args.no_cpu_baseline:
            st = solver.symbolic_stats(0)
            cpu = cpu_baseline_sample(RPMS[1], st["flops"])
        line = {
            "metric": METRIC, "value": tot_ok / t_dev if t_dev > 0 else 0.0, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / max(len(timed), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "harmonics": args.harmonics, "num_modes": args.num_modes,
                       "speeds": [float(r) for r in timed], "parallelism": f"replicas x{ws} (speeds sharded)",
                       "l2": "inputs larger than L2 (no flush needed)"},
            "eigenpairs": {"verified": int(tot_ok), "returned": int(tot_all), "worst_rel_err_vs_fp64": worst,
                           "distinct_verified": int(tot_distinct) if n_distinct is not None else None},
            "fp64_gpu": {"value": fp64_pairs / (fp64_ms / 1e3) if fp64_ms > 0 else None, "unit": UNIT,
                         "ms_per_step": fp64_ms / max(len(timed), 1)},
            "e2e": {"value": tot_ok / t_wall if t_wall > 0 else 0.0, "unit": UNIT,
                    "h2d_bytes_per_step": 8 + 4 * max(len(hi), 19), "d2h_bytes_per_step": int(d2h / max(len(timed), 1))},
            "gpu_launches": launches,
            "roofline": {"kernel": f"shift-invert triangular solve of the {len(mesh_k)} complex harmonics "
                                   "(supernodal sweeps, one CUDA graph per batched solve)",
                         "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak if hbm_peak else None, "traffic": traffic,
                         "per_launch_bytes": per_launch_bytes, "launches": prof["count"],
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback"},
            "cpu_baseline": cpu,
            "serving": serving,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
