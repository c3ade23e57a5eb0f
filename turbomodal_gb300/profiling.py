"""Fixed workloads for profiler captures of the GPU path.

``python -m turbomodal_gb300.profiling <case> [reps] [tensor_cores]`` solves the complex
harmonics of one sector at 10000 rpm in mixed precision ``reps`` times and prints the per-call
timing, then solves once more with every batched triangular solve timed by CUDA events and
prints their mean time and algorithmic bandwidth; ``tensor_cores`` (0 or 1) sets the
factorisation's trailing-update path (default: the library's) and ``autotune`` (0 or 1) the
supernode-shape autotuner (with ``TMG_VERBOSE=1`` set it prints every candidate's factorisation
and all-problems triangular-solve time).  Cases:

* ``medium``  — 11,305-node bladed sector (20x12x4 hub + 16x6x2 blade, 36 sectors, n = 32,160
  free DOF per harmonic, 17 complex harmonics in one batch): small enough for multi-pass
  profiler captures (a few GB on the device) while its factors are larger than L2.
* ``config1`` — the 57,897-node config-1 sector of the benchmark (n = 168,660).
"""

from __future__ import annotations

import sys
import time

from .meshgen import TITANIUM, config_mesh, sector_mesh
from .solver import CyclicSymmetrySolver


def case_mesh(name: str):
    if name == "config1":
        return config_mesh(1)
    if name == "medium":
        return sector_mesh(20, 12, 4, num_sectors=36, jitter=0.02, seed=7,
                           blade=dict(ns=16, nc=6, nb=2, span=0.12, chord=0.05, thick=0.004, twist_deg=30.0))
    raise ValueError(f"unknown case {name!r}")


def main(argv: list[str]) -> None:
    name = argv[0] if argv else "medium"
    reps = int(argv[1]) if len(argv) > 1 else 1
    mesh = case_mesh(name)
    solver = CyclicSymmetrySolver(mesh, TITANIUM)
    if len(argv) > 2:
        solver.set_option("tensor_cores", float(argv[2]))
    if len(argv) > 3:
        solver.set_option("autotune", float(argv[3]))
    ks = list(range(1, mesh.num_sectors // 2))
    for r in range(reps):
        t = time.time()
        res = solver.solve_at_rpm(10000.0, 10, harmonic_indices=ks, precision="mixed")
        print(f"{name} rep {r}: {len(res)} results {time.time() - t:.2f} s {solver.last_timing()}", flush=True)
    # one more call with every batched triangular solve timed by CUDA events
    solver.set_profiling(True)
    solver.solve_at_rpm(10000.0, 10, harmonic_indices=ks, precision="mixed")
    prof = solver.profile_solve()
    solver.set_profiling(False)
    ms = prof["ms"] / max(prof["count"], 1)
    gbs = prof["bytes"] / max(prof["count"], 1) / (ms * 1e-3) / 1e9
    print(f"{name} triangular solves: {prof['count']} x {ms:.3f} ms, {gbs:.0f} GB/s algorithmic", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
