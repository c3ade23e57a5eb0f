#!/usr/bin/env python
"""Benchmark: converged eigenpairs/s of the cyclic-symmetry modal solve on GB300.

Workload: the batched rpm sweep on the rotating bladed-disk sector (config-1 mesh:
40x24x6 hub + 30x10x2 twisted blade, 57,897 nodes, titanium, 36 sectors), 24 speeds in
linspace(0, 15000) rpm x harmonic indices 0..18, num_modes = 10, rotating effects (spin
softening + stress stiffening), standard Hermitian shift-invert path.  A step is one speed
of the sweep (all 19 harmonic problems: assembly, prestress, projections, factorisations,
Lanczos, expansion).  Speeds are taken in order, --sweep-group of them per solve_rpm_sweep
call (their harmonics are factorised and iterated as one batch; each speed is charged an equal
share of the call).  Rank r of N takes speeds r, r+N, ... (weak scaling: per-GPU work fixed).

value   eigenpairs/s of the mixed path (FP32 LDL^H + FP64 refinement), counting the eigenpairs
        that converged and lie within 1e-6 relative frequency error of the plain FP64 GPU path,
        on --verify-steps timed speeds spread over the sweep (re-solved in FP64 after the timed
        region), over those speeds' device time (CUDA events on the library's stream).
e2e     the same count over the wall-clock of the public API call (solve_rpm_sweep through the
        C ABI: speeds and harmonic list in, frequencies, mode shapes and modal masses copied back
        to host).
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
METRIC = "converged eigenpairs/s @1e-6 rel freq err, config-1 bladed-disk rpm sweep"
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
    ap.add_argument("--verify-steps", type=int, default=4,
                    help="timed speeds (spread over the sweep) re-solved on the plain FP64 GPU path")
    ap.add_argument("--wall-budget", type=float, default=1200.0,
                    help="seconds after start beyond which the optional legs (serving sample, CPU baseline) "
                         "are skipped")
    ap.add_argument("--refine-tol", type=float, default=1e-8,
                    help="relative residual target of the FP64 refinement of every mixed solve (frequencies are "
                         "still verified against the FP64 path at 1e-6)")
    ap.add_argument("--sweep-group", type=int, default=2,
                    help="speeds per solve_rpm_sweep call (their harmonics are factorised and iterated as one batch)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the served request-stream sample")
    ap.add_argument("--serve-requests", type=int, default=16)
    ap.add_argument("--serve-max-nodes", type=int, default=200000,
                    help="largest sector of the request-stream sample")
    ap.add_argument("--serve-deadline", type=float, default=180.0,
                    help="no served batch starts later than this many seconds into the stream")
    ap.add_argument("--serve-designs", type=int, default=4,
                    help="distinct sector designs the requests draw from (repeats are batched and reuse contexts)")
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


def mem_available_bytes() -> int:
    """Host memory this process may still use: MemAvailable, capped by the cgroup limit."""
    avail = 8 << 30
    try:
        with open("/proc/meminfo") as fh:
            for line in fh:
                if line.startswith("MemAvailable:"):
                    avail = int(line.split()[1]) * 1024
    except OSError:
        pass
    for lim, use in (("/sys/fs/cgroup/memory.max", "/sys/fs/cgroup/memory.current"),
                     ("/sys/fs/cgroup/memory/memory.limit_in_bytes", "/sys/fs/cgroup/memory/memory.usage_in_bytes")):
        try:
            with open(lim) as fh:
                raw = fh.read().strip()
            if raw == "max":
                continue
            with open(use) as fh:
                used = int(fh.read().strip())
            avail = min(avail, max(0, int(raw) - used))
        except (OSError, ValueError):
            continue
    return avail


class ReferenceSample:
    """The reference's CPU path for one speed of the config-1 sweep, measured on the config-1
    operator itself in bounded samples (the oracle restates it; the reference needs Eigen and
    Spectra, which cannot be built here).

    Per speed the reference assembles and projects the sector, then solves the 19 harmonics on
    a std::thread pool (src/cyclic_solver.cpp:1226-1332): for each, Eigen's up-looking
    SimplicialLDLT of K_k - M_k and the shift-invert Lanczos.  One factorisation of the config-1
    operator takes ~20 min on one core, so it is measured in row windows
    (oracle/orc_window.hpp): the rows are cut into W windows of equal loop work, and every
    sample runs one window of the numeric loop on the real structure of L, `threads` windows at
    once on separate threads (each its own copy of L, as the pool runs one harmonic per thread),
    each followed by one whole triangular solve.  Estimates:
      T_fact  = W x mean window time   (every window has the same work)
      T_harm  = T_fact + 40 x T_solve  (ncv = 40 shift-invert applications; no restarts)
      T_speed = T_prep + (17 T_harm + 2 T_harm / 4) / threads
    T_prep is the oracle's assembly and cyclic projections at rest, timed once.  Left out, which
    favours the CPU: the prestress solve at speed, Lanczos restarts and reorthogonalisation,
    M products; the real harmonics k = 0, 18 are counted at a quarter of a complex one, and the
    pool at perfect load balance."""

    PAIRS_PER_SPEED = 190     # 19 harmonics x 10 modes, as the GPU arm counts them

    def __init__(self, threads: int | None = None, target_window_s: float = 4.0, planned_samples: int = 0,
                 mesh=None):
        from oracle import orc
        from turbomodal_gb300.meshgen import TITANIUM, config_mesh

        orc.build()
        t0 = time.perf_counter()
        self.mesh = mesh if mesh is not None else config_mesh(1)
        om = orc.OracleModel(self.mesh, TITANIUM)
        om.prepare(0.0)
        self.t_prep = time.perf_counter() - t0
        A = (om.matrix("Kk", k=1) - om.matrix("Mk", k=1)).tocsc()
        del om
        self.lw = orc.LdlWindows(A)
        self.n = self.lw.n
        slot_bytes = 16 * self.lw.nnz_l + 64 * self.n
        want = threads or os.cpu_count() or 1
        fit = max(1, int(0.6 * mem_available_bytes() // slot_bytes))
        self.threads = max(1, min(want, 17, fit))
        for _ in range(self.threads - 1):
            self.lw.add_slot()
        self.cum = self.lw.cumwork()
        # probe: one window of 1/4000 of the loop work on one thread sets the window count
        b = int(np.searchsorted(self.cum, self.cum[-1] / 4000.0))
        tf, _ = self.lw.run([0], [0], [max(b, 1)], solve=False)
        est = max(tf[0], 1e-6) * 4000.0
        self.W = max(1, planned_samples, int(round(est / target_window_s)))
        self.bnd = np.searchsorted(self.cum, np.linspace(0, self.cum[-1], self.W + 1))
        self.bnd[0], self.bnd[-1] = 0, self.n
        self.planned = max(1, planned_samples)
        self.next = 0
        self.t_fact, self.t_solve = [], []
        self.setup_s = time.perf_counter() - t0

    def step(self, record: bool = True) -> float:
        """One sample round: `threads` windows at once, each followed by one solve; returns its
        wall time."""
        idx = [(self.next + t) % self.planned for t in range(self.threads)]
        if record:
            self.next += self.threads
        win = [min(self.W - 1, int((q + 0.5) * self.W / self.planned)) for q in idx]
        a = [int(self.bnd[w]) for w in win]
        b = [int(self.bnd[w + 1]) for w in win]
        t0 = time.perf_counter()
        tf, ts = self.lw.run(list(range(self.threads)), a, b, solve=True)
        dt = time.perf_counter() - t0
        if record:
            self.t_fact += list(tf)
            self.t_solve += list(ts)
        return dt

    def estimate(self) -> dict:
        t_fact = self.W * float(np.mean(self.t_fact))
        t_solve = float(np.mean(self.t_solve))
        t_harm = t_fact + 40.0 * t_solve
        t_speed = self.t_prep + (17.0 * t_harm + 2.0 * t_harm / 4.0) / self.threads
        return {"value": self.PAIRS_PER_SPEED / t_speed, "t_speed_s": t_speed, "t_fact_s": t_fact,
                "t_solve_s": t_solve, "t_prep_s": self.t_prep}

    def describe(self, sampled_s: float) -> str:
        e = self.estimate()
        return (f"oracle (Eigen SimplicialLDLT + Lanczos restated) on the config-1 harmonic operator "
                f"(n={self.n}, nnz(L)={self.lw.nnz_l}): {len(self.t_fact)} of {self.W} equal-work row windows "
                f"of the up-looking LDL^H timed, {self.threads} at once on {self.threads} threads, plus "
                f"{len(self.t_solve)} whole solves ({sampled_s:.0f} s sampled); per harmonic factor "
                f"{e['t_fact_s']:.0f} s + 40 solves x {e['t_solve_s']:.2f} s, assembly+projections "
                f"{e['t_prep_s']:.0f} s; one speed = {e['t_speed_s']:.0f} s on {self.threads} threads "
                f"(prestress solve, restarts and reorthogonalisation left out, real harmonics at 1/4)")


def cpu_baseline_sample(threads: int | None = None, windows: int = 2):
    """The GPU arm's cpu_baseline: a short ReferenceSample (`windows` sample rounds)."""
    rs = ReferenceSample(threads=threads, planned_samples=windows * (threads or os.cpu_count() or 1))
    t0 = time.perf_counter()
    for _ in range(windows):
        rs.step()
    sampled = time.perf_counter() - t0
    e = rs.estimate()
    return {"value": e["value"], "unit": UNIT, "cores": rs.threads, "kind": "port",
            "sample": rs.describe(sampled), "sample_seconds": sampled + rs.setup_s}


def run_reference(args, ws, rank, pg):
    """Reference arm: the reference's CPU algorithm (the oracle restatement; the reference itself
    needs Eigen and Spectra, which are not available) on the config-1 sweep, sampled as
    ReferenceSample describes: every timed step is one round of concurrent row windows, and the
    line's value is the eigenpairs/s of one speed estimated from all timed rounds."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    rs = ReferenceSample(threads=cores, planned_samples=args.steps * min(cores, 17))
    log(f"reference sample: setup {rs.setup_s:.1f} s, {rs.threads} threads, {rs.W} windows")
    for i in range(args.warmup):
        rs.step(record=False)
    step_s = []
    for i in range(args.steps):
        step_s.append(rs.step())
        log(f"reference step {i + 1}/{args.steps}: {step_s[-1]:.1f} s")
    e = rs.estimate()
    v = e["value"]
    ms = 1e3 * float(np.mean(step_s))
    sample = rs.describe(sum(step_s))
    line = {"impl": "reference",
            "metric": METRIC,
            "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "path": "reference CPU path (oracle): simplicial LDL^H + Lanczos, FP64, "
                                                     f"{rs.threads} host threads",
                       "l2": "inputs larger than L2",
                       "step": "one round of concurrent row-window samples of the config-1 factorisation"},
            "reference_estimate": e,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": rs.threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


T_START = time.perf_counter()


def log(msg: str) -> None:
    """Progress on stderr (the JSON line alone goes to stdout)."""
    sys.stderr.write(f"[bench {time.perf_counter() - T_START:7.1f} s] {msg}\n")
    sys.stderr.flush()


def verify_indices(n_timed: int, n_verify: int) -> list[int]:
    """Timed steps re-solved on the FP64 path: n_verify of them spread evenly over the sweep
    (first and last included)."""
    if n_timed <= 0 or n_verify <= 0:
        return []
    return sorted({int(round(x)) for x in np.linspace(0, n_timed - 1, min(n_verify, n_timed))})


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
    # deflated refinement (previous speed's eigenvectors); SIMT trailing updates (the library
    # default); supernode shapes tuned on the first batch of each operator pattern (at rest and
    # at speed, both in the warm-up speeds)
    solver = CyclicSymmetrySolver(mesh, TITANIUM, device=local, precision="mixed", deflate=True)
    solver.set_option("refine_tol", args.refine_tol)
    solver.set_option("autotune", 1)
    order = list(my_rpms) * (1 + (args.warmup + args.steps) // max(1, len(my_rpms)))
    warm, timed = order[: args.warmup], order[args.warmup: args.warmup + args.steps]
    grp = max(1, args.sweep_group)
    log(f"config-1 mesh {mesh.num_nodes()} nodes; {len(warm)} warm-up and {len(timed)} timed speeds, "
        f"{grp} speeds per sweep call")
    for c0 in range(0, len(warm), grp):
        t0 = time.perf_counter()
        solver.solve_rpm_sweep(warm[c0:c0 + grp], args.num_modes, hi, precision="mixed")
        log(f"warm-up speeds {c0 + 1}-{min(len(warm), c0 + grp)}/{len(warm)}: {time.perf_counter() - t0:.1f} s")
    torch.cuda.synchronize()
    barrier(pg)
    clocks = ClockSampler(local)
    clocks.start()
    dev_ms, wall_s, results, launches, d2h = [], [], [], 0, []
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    for c0 in range(0, len(timed), grp):
        chunk = timed[c0:c0 + grp]
        t0 = time.perf_counter()
        sweep = solver.solve_rpm_sweep(chunk, args.num_modes, hi, precision="mixed")
        w = time.perf_counter() - t0
        tm = solver.last_timing()
        launches += int(tm["kernel_launches"])
        for res in sweep:   # each speed of the call gets an equal share of its time
            wall_s.append(w / len(chunk))
            dev_ms.append(tm["device_ms"] / len(chunk))
            d2h.append(sum(r.frequencies.nbytes + r.mode_shapes.nbytes + r.whirl_direction.nbytes +
                           r.modal_mass_kg.nbytes for r in res))
            results.append(res)
        log(f"timed speeds {c0 + 1}-{c0 + len(chunk)}/{len(timed)} ({', '.join(f'{r:.0f}' for r in chunk)} rpm): "
            f"{tm['device_ms'] / 1e3:.2f} s device, {w:.2f} s wall, "
            f"{sum(len(r.frequencies) for res in sweep for r in res)} eigenpairs")
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    barrier(pg)
    # verification of a stated subset of the timed speeds against the plain FP64 GPU path
    # (untimed); value and e2e count the verified eigenpairs of exactly those speeds
    vidx = [] if args.no_verify else verify_indices(len(timed), args.verify_steps)
    n_ok = n_all = n_distinct = 0
    worst = 0.0
    fp64_ms, fp64_pairs = 0.0, 0
    for q, i in enumerate(vidx):
        ref = solver.solve_at_rpm(timed[i], args.num_modes, hi, precision="fp64")
        fp64_ms += solver.last_timing()["device_ms"]
        fp64_pairs += sum(len(r.frequencies) for r in ref if r.converged)
        a, b, w = count_verified(results[i], ref)
        n_ok += a
        n_all += b
        n_distinct += count_distinct_verified(results[i], ref)
        worst = max(worst, w)
        log(f"verified {q + 1}/{len(vidx)} at {timed[i]:.0f} rpm: {a}/{b} within 1e-6 (worst {w:.2e})")
    if args.no_verify:   # unverified run: every returned eigenpair of every timed speed
        vidx = list(range(len(timed)))
        n_ok = n_all = sum(len(r.frequencies) for res in results for r in res)
    v_dev_s = sum(dev_ms[i] for i in vidx) / 1e3
    v_wall_s = sum(wall_s[i] for i in vidx)
    # roofline of the dominant kernel: the shift-invert triangular-solve graph of the batch of
    # complex harmonics (HBM bound), timed live with CUDA events in one extra profiled sweep call
    # of the timed batch shape (the complex harmonics of --sweep-group speeds)
    mesh_k = [k for k in (hi or range(mesh.num_sectors // 2 + 1)) if 0 < k < mesh.num_sectors / 2]
    solver.set_profiling(True)
    solver.solve_rpm_sweep(timed[:grp], args.num_modes, mesh_k, precision="mixed")
    prof = solver.profile_solve()
    solver.set_profiling(False)
    log(f"profiled solve: {prof['count']} batched triangular solves, {prof['ms']:.1f} ms")
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
    traffic = None   # DRAM bytes of one batched solve: the ncu-measured DRAM / algorithmic ratio
    tr_path = os.path.join(ROOT, "profiles", "trisolve_cfg1_traffic.txt")
    if os.path.exists(tr_path):
        with open(tr_path) as fh:
            for line in fh:
                if line.startswith("dram_over_algorithmic"):
                    traffic = float(line.split("=")[1]) * per_launch_bytes
    t_dev_all = max_over_ranks(pg, sum(dev_ms) / 1e3)
    tune_rows = solver.tuning_report()
    t_dev = max_over_ranks(pg, v_dev_s)
    t_wall = max_over_ranks(pg, v_wall_s)
    tot_ok = sum_over_ranks(pg, n_ok)
    tot_all = sum_over_ranks(pg, n_all)
    tot_distinct = sum_over_ranks(pg, n_distinct)
    tot_returned = sum_over_ranks(pg, sum(len(r.frequencies) for res in results for r in res))
    skipped = []
    serving = None
    if rank == 0 and not args.no_serve:
        if time.perf_counter() - T_START > args.wall_budget:
            skipped.append("serving")
        else:
            # served request stream (Poisson arrivals, mixed sizes, admission by memory budget)
            from turbomodal_gb300.serve import ModalServer, latency_summary, request_stream

            reqs = request_stream(args.serve_requests, seed=2024, rate_hz=20.0, min_nodes=2000,
                                  max_nodes=args.serve_max_nodes, distinct_sectors=args.serve_designs)
            srv = ModalServer(device=local, budget_bytes=150 << 30, max_inflight=4)
            done = srv.serve(reqs, deadline_s=args.serve_deadline)
            srv.close()
            serving = latency_summary(done)
            serving["deadline_s"] = args.serve_deadline
            sizes = sorted({r.mesh.num_nodes() for r in reqs})
            serving["sample"] = (f"{len(reqs)} requests, Poisson 20 req/s, drawn from {args.serve_designs} config-0/1-"
                                 f"style sector designs ({', '.join(str(n) for n in sizes)} nodes; log-uniform in "
                                 f"2000-{args.serve_max_nodes}), 24/36/48 sectors, rpm U(0,15000), 5-20 modes, 1-19 "
                                 "random harmonics, mixed precision, 150 GB budget, 4 in flight, same-sector "
                                 "requests batched")
            log(f"serving sample: p50 {serving.get('p50_s')} s, p99 {serving.get('p99_s')} s")
    if rank == 0:
        cpu = None
        if ws == 1 and not args.no_cpu_baseline:
            if time.perf_counter() - T_START > args.wall_budget:
                skipped.append("cpu_baseline")
            else:
                cpu = cpu_baseline_sample(threads=None, windows=2)
                log(f"cpu baseline: {cpu['value']:.4g} eigenpairs/s ({cpu['sample_seconds']:.1f} s sampled)")
        line = {
            "metric": METRIC, "value": tot_ok / t_dev if t_dev > 0 else 0.0, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev_all / max(len(timed), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "path": "mixed FP32 supernodal LDL^H + FP64 refinement, 1 GB300",
                       "harmonics": args.harmonics, "num_modes": args.num_modes,
                       "speeds": [float(r) for r in timed], "speeds_per_call": grp,
                       "deflated_refinement": True, "tensor_core_updates": bool(solver.get_option("tensor_cores")),
                       "supernode_autotune": True,
                       "supernode_shape": next(({"relax": r["relax"], "max_width": int(r["max_width"]),
                                                 "solve_ms": round(r["solve_ms"], 2), "factor_ms": round(r["factor_ms"], 1)}
                                                for r in tune_rows if r["chosen"]), None),
                       "refine_tol": args.refine_tol,
                       "verified_speeds": [float(timed[i]) for i in vidx],
                       "parallelism": f"replicas x{ws} (speeds sharded)",
                       "l2": "inputs larger than L2 (no flush needed)"},
            "eigenpairs": {"verified": int(tot_ok), "returned_on_verified_speeds": int(tot_all),
                           "returned_all_speeds": int(tot_returned), "worst_rel_err_vs_fp64": worst,
                           "distinct_verified": int(tot_distinct),
                           "returned_per_s_all_speeds": tot_returned / t_dev_all if t_dev_all > 0 else None},
            "fp64_gpu": {"value": fp64_pairs / (fp64_ms / 1e3) if fp64_ms > 0 else None, "unit": UNIT,
                         "ms_per_step": fp64_ms / max(len(vidx), 1), "speeds": len(vidx) if not args.no_verify else 0},
            "e2e": {"value": tot_ok / t_wall if t_wall > 0 else 0.0, "unit": UNIT,
                    "h2d_bytes_per_step": 8 + 4 * max(len(hi), 19) // grp,
                    "d2h_bytes_per_step": int(np.mean(d2h)) if d2h else 0},
            "gpu_launches": launches,
            "roofline": {"kernel": f"shift-invert triangular solve of the {len(mesh_k)} complex harmonics of "
                                   f"{min(grp, len(timed))} speeds (supernodal sweeps, one CUDA graph per batched solve)",
                         "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak if hbm_peak else None, "traffic": traffic,
                         "per_launch_bytes": per_launch_bytes, "launches": prof["count"],
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback"},
            "cpu_baseline": cpu,
            "serving": serving,
            "skipped": skipped,
            "clocks": clk,
        }
        if line["fp64_gpu"]["value"]:
            line["mixed_over_fp64_gpu"] = line["value"] / line["fp64_gpu"]["value"]
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
