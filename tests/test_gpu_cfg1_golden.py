"""Config-1 bladed-disk sector (57,897 nodes) at 10000 rpm against the FP64 oracle.

The oracle (CPU restatement of the reference path: assembly, prestress, projections,
simplicial LDL^H and Hermitian Lanczos) takes about an hour on this sector, so its result for
harmonics 0, 1, 9 and 18 (10 modes) is a committed fixture, tests/golden/cfg1_rpm10000.npz,
made by tests/golden/make_cfg1_golden.py.  The fixture keeps the mode shapes on a seeded
sample of 2048 sector DOFs; the test compares, for both precisions of the GPU path:
frequencies within 1e-6 relative, whirl directions equal, and the subspace MAC on the sampled
rows >= 0.999 (degenerate pairs and near-coincident modes compared as subspaces).
"""

import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FREQ_TOL = 1e-6
MAC_MIN = 0.999
PATH = os.path.join(GOLDEN, "cfg1_rpm10000.npz")


def subspace_mac(phi, Psi):
    Q, _ = np.linalg.qr(Psi)
    v = Q.conj().T @ phi
    return float(np.real(np.vdot(v, v)) / np.real(np.vdot(phi, phi)))


@pytest.fixture(scope="module")
def golden():
    if not os.path.exists(PATH):
        pytest.fail("missing fixture tests/golden/cfg1_rpm10000.npz (run tests/golden/make_cfg1_golden.py)")
    return np.load(PATH)


@pytest.fixture(scope="module")
def solver():
    from turbomodal_gb300.meshgen import TITANIUM, config_mesh
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    return CyclicSymmetrySolver(config_mesh(1), TITANIUM)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_config1_matches_oracle_fixture(golden, solver, precision):
    ks = [int(k) for k in golden["k"]]
    dofs = golden["dofs"]
    res = {r.harmonic_index: r for r in solver.solve_at_rpm(float(golden["rpm"]), int(golden["num_modes"]), ks,
                                                             precision=precision)}
    assert sorted(res) == sorted(ks)
    for k in ks:
        r = res[k]
        f, w, shp = golden[f"freq_{k}"], golden[f"whirl_{k}"], golden[f"shape_{k}"]
        assert r.converged == bool(golden[f"conv_{k}"])
        assert len(r.frequencies) == len(f), k
        err = np.abs(r.frequencies - f) / f
        assert err.max() <= FREQ_TOL, (k, precision, err.max())
        assert np.array_equal(r.whirl_direction, w)
        for q in range(len(f)):
            cluster = np.abs(f - r.frequencies[q]) <= 1e-6 * r.frequencies[q]
            assert subspace_mac(r.mode_shapes[dofs, q], shp[:, cluster]) >= MAC_MIN, (k, q, precision)
