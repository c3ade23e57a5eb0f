"""Tensor-core (tcgen05, three-way BF16 split) trailing Schur updates of the mixed path's complex FP32
factorisation against the same factorisation on the FP32 SIMT pipe.

Both factors only precondition the FP64-refined shift-invert solves, which stop at a 1e-10
relative residual, so the frequencies must agree within 1e-9 relative and the modes at
MAC >= 0.999.  The quality of the factor shows in the refinement: with the tensor-core
updates the most refinement iterations of one application may exceed the SIMT factor's by at
most 2, and the total number of FP32 solves by at most 25 %.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FREQ_TOL = 1e-9
MAC_MIN = 0.999


def subspace_mac(phi, Psi):
    Q, _ = np.linalg.qr(Psi)
    v = Q.conj().T @ phi
    return float(np.real(np.vdot(v, v)) / np.real(np.vdot(phi, phi)))


@pytest.mark.parametrize("mesh_args", [dict(cfg=0), dict(nodes=20000)])
def test_tensor_core_factor_matches_simt_factor(mesh_args):
    from turbomodal_gb300.meshgen import TITANIUM, config_mesh, scaled_mesh
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    m = config_mesh(0) if "cfg" in mesh_args else scaled_mesh(mesh_args["nodes"], 36, seed=5)
    simt = CyclicSymmetrySolver(m, TITANIUM, precision="mixed")
    tc = CyclicSymmetrySolver(m, TITANIUM, precision="mixed")
    assert tc.get_option("tensor_cores") == 0.0   # the SIMT updates are the default
    tc.set_option("tensor_cores", 1)
    ks = [1, 2, 9, 17]
    a = {r.harmonic_index: r for r in simt.solve_at_rpm(9000.0, 10, harmonic_indices=ks)}
    ta = simt.last_timing()
    b = {r.harmonic_index: r for r in tc.solve_at_rpm(9000.0, 10, harmonic_indices=ks)}
    tb = tc.last_timing()
    assert sorted(a) == sorted(b) == ks
    for k in ks:
        fa, fb = a[k].frequencies, b[k].frequencies
        assert len(fa) == len(fb)
        assert np.max(np.abs(fa - fb) / fa) <= FREQ_TOL, k
        assert b[k].refine_residual <= 1e-10
        for q in range(len(fb)):
            cluster = np.abs(fa - fb[q]) <= 1e-6 * fb[q]
            assert subspace_mac(b[k].mode_shapes[:, q], a[k].mode_shapes[:, cluster]) >= MAC_MIN
    assert tb["max_refine_iters"] <= ta["max_refine_iters"] + 2, (ta, tb)
    assert tb["solves"] <= 1.25 * ta["solves"], (ta, tb)
