"""Batched rpm sweep (tmg_solve_sweep: the harmonics of several speeds factorised and iterated as
one batch) against one tmg_solve_at_rpm per speed, the reference's loop
(src/cyclic_solver.cpp:1359-1373).

Every problem of a batch runs its own factorisation, refinement and Lanczos iteration (the batch
only shares launches), so each speed's frequencies must equal the per-speed solve's within
1e-9 relative for both precisions, with the same harmonics, whirl directions and modal masses
(1e-9), and modes at MAC >= 0.999.  The sweep mixes rest (its own operator pattern) and speed.
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


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("mesh_args", [dict(cfg=0), dict(nodes=20000)])
def test_sweep_equals_per_speed_solves(mesh_args, precision):
    from turbomodal_gb300.meshgen import TITANIUM, config_mesh, scaled_mesh
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    m = config_mesh(0) if "cfg" in mesh_args else scaled_mesh(mesh_args["nodes"], 36, seed=5)
    rpms = [0.0, 4000.0, 8000.0, 12000.0]
    ks = [0, 1, 5, 18] if "cfg" in mesh_args else []
    sweep = CyclicSymmetrySolver(m, TITANIUM, precision=precision).solve_rpm_sweep(rpms, 6, ks)
    single = CyclicSymmetrySolver(m, TITANIUM, precision=precision)
    assert len(sweep) == len(rpms)
    for rpm, res in zip(rpms, sweep):
        ref = single.solve_at_rpm(rpm, 6, ks)
        assert [r.harmonic_index for r in res] == [r.harmonic_index for r in ref]
        for a, b in zip(res, ref):
            assert a.rpm == rpm and len(a.frequencies) == len(b.frequencies)
            assert np.max(np.abs(a.frequencies - b.frequencies) / b.frequencies) <= FREQ_TOL, (rpm, a.harmonic_index)
            assert np.array_equal(a.whirl_direction, b.whirl_direction)
            np.testing.assert_allclose(a.modal_mass_kg, b.modal_mass_kg, rtol=1e-9)
            for q in range(len(a.frequencies)):
                cluster = np.abs(b.frequencies - a.frequencies[q]) <= 1e-6 * a.frequencies[q]
                assert subspace_mac(a.mode_shapes[:, q], b.mode_shapes[:, cluster]) >= MAC_MIN


def test_rpm_sweep_module_function_uses_the_batched_sweep(cfg0_mesh):
    from turbomodal_gb300.meshgen import TITANIUM
    from turbomodal_gb300.solver import CyclicSymmetrySolver, rpm_sweep

    out = rpm_sweep(cfg0_mesh, TITANIUM, [2000.0, 6000.0], 4, harmonic_indices=[0, 3], precision="mixed")
    s = CyclicSymmetrySolver(cfg0_mesh, TITANIUM, precision="mixed")
    for rpm, res in zip([2000.0, 6000.0], out):
        ref = s.solve_at_rpm(rpm, 4, [0, 3])
        for a, b in zip(res, ref):
            np.testing.assert_allclose(a.frequencies, b.frequencies, rtol=FREQ_TOL)
            assert np.all(a.modal_mass_kg > 0)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_returning_to_rest_reuses_the_kept_pattern_state(cfg0_mesh, precision):
    """Rest and speed have different operator patterns; the context keeps the other regime's
    unions and symbolic analyses, so a sweep that goes rest -> speed -> rest -> speed reuses them.
    Every speed's result equals a fresh solver's within 1e-9."""
    from turbomodal_gb300.meshgen import TITANIUM
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    rpms = [0.0, 5000.0, 0.0, 9000.0]
    s = CyclicSymmetrySolver(cfg0_mesh, TITANIUM, precision=precision)
    seq = [s.solve_rpm_sweep([r], 5, [0, 2, 18])[0] for r in rpms]
    for rpm, res in zip(rpms, seq):
        fresh = CyclicSymmetrySolver(cfg0_mesh, TITANIUM, precision=precision).solve_at_rpm(rpm, 5, [0, 2, 18])
        assert [r.harmonic_index for r in res] == [r.harmonic_index for r in fresh]
        for a, b in zip(res, fresh):
            np.testing.assert_allclose(a.frequencies, b.frequencies, rtol=FREQ_TOL)
