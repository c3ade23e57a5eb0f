"""Deflated refinement CG of the mixed path (TMG_OPT_DEFLATE) against the undeflated path.

Deflation changes only how each FP64-refined shift-invert solve reaches its 1e-10 residual
target (the CG starts in, and is projected against, the span of the previous speed's lowest
eigenvectors), so every frequency must equal the undeflated result within 1e-9 relative and
every mode must match at MAC >= 0.999.  The test also checks that the deflated sweep does not
need more FP32 triangular solves than the undeflated one.
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
def test_deflated_refinement_equals_undeflated(mesh_args):
    from turbomodal_gb300.meshgen import TITANIUM, config_mesh, scaled_mesh
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    m = config_mesh(0) if "cfg" in mesh_args else scaled_mesh(mesh_args["nodes"], 36, seed=5)
    plain = CyclicSymmetrySolver(m, TITANIUM, precision="mixed")
    defl = CyclicSymmetrySolver(m, TITANIUM, precision="mixed", deflate=True)
    assert defl.get_option("deflate") == 1.0 and plain.get_option("deflate") == 0.0
    solves = {"plain": 0, "defl": 0}
    for rpm in (6000.0, 7000.0, 8000.0):
        a = {r.harmonic_index: r for r in plain.solve_at_rpm(rpm, 10)}
        solves["plain"] += plain.last_timing()["solves"]
        b = {r.harmonic_index: r for r in defl.solve_at_rpm(rpm, 10)}
        solves["defl"] += defl.last_timing()["solves"]
        assert sorted(a) == sorted(b)
        for k in a:
            fa, fb = a[k].frequencies, b[k].frequencies
            assert len(fa) == len(fb)
            assert np.max(np.abs(fa - fb) / fa) <= FREQ_TOL, (rpm, k)
            assert b[k].refine_residual <= 1e-10
            for q in range(len(fb)):
                cluster = np.abs(fa - fb[q]) <= 1e-6 * fb[q]
                assert subspace_mac(b[k].mode_shapes[:, q], a[k].mode_shapes[:, cluster]) >= MAC_MIN
    assert solves["defl"] <= solves["plain"], solves
