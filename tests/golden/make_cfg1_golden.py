"""Generate the config-1 parity fixture from the oracle (CPU restatement of the reference path).

Config-1 bladed-disk sector (40x24x6 hub + 30x10x2 twisted blade, 57,897 nodes, titanium,
36 sectors) at 10000 rpm with stress stiffening and spin softening, 10 modes, harmonic
indices 0, 1, 9 and 18, all in FP64 on the host: assembly, prestress solve, cyclic
projections, simplicial LDL^H shift-invert and the Hermitian Lanczos of the reference
(src/cyclic_solver.cpp:725-1357).  The run takes about an hour of host time (four
harmonics on four threads; each complex factorisation is ~3e12 flops).

Stored in tests/golden/cfg1_rpm10000.npz:
  k, frequencies (per k), whirl, converged, iterations;
  dofs: a seeded sample of 2048 full-sector DOF indices, and the mode shapes restricted to
  those rows (the full shapes are 174k x 10 complex per harmonic, too large for a fixture).
The GPU test compares frequencies within 1e-6 and the subspace MAC on the sampled rows.

Usage:  python tests/golden/make_cfg1_golden.py [threads]
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

RPM = 10000.0
KS = [0, 1, 9, 18]
NUM_MODES = 10
N_SAMPLE = 2048
OUT = os.path.join(HERE, "cfg1_rpm10000.npz")


def main(threads: int) -> None:
    from oracle import orc
    from turbomodal_gb300.meshgen import TITANIUM, config_mesh

    orc.build()
    m = config_mesh(1)
    t0 = time.time()
    om = orc.OracleModel(m, TITANIUM)
    om.prepare(RPM)
    print(f"prepare {time.time() - t0:.1f} s", flush=True)
    t1 = time.time()
    res = om.solve(RPM, NUM_MODES, harmonic_indices=KS, max_threads=threads, with_shapes=True)
    print(f"solve {time.time() - t1:.1f} s", flush=True)
    rng = np.random.default_rng(20261204)
    dofs = np.sort(rng.choice(m.num_dof(), size=N_SAMPLE, replace=False)).astype(np.int64)
    out = {"dofs": dofs, "rpm": np.float64(RPM), "num_modes": np.int32(NUM_MODES),
           "num_nodes": np.int32(m.num_nodes())}
    ks = []
    for r in sorted(res, key=lambda r: r["harmonic_index"]):
        k = r["harmonic_index"]
        ks.append(k)
        out[f"freq_{k}"] = r["frequencies"]
        out[f"whirl_{k}"] = r["whirl_direction"].astype(np.int32)
        out[f"conv_{k}"] = np.int32(r["converged"])
        out[f"iter_{k}"] = np.int32(r["iterations"])
        out[f"shape_{k}"] = r["mode_shapes"][dofs, :]
        print(k, r["converged"], r["iterations"], r["frequencies"], flush=True)
    out["k"] = np.asarray(ks, np.int32)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 4)
