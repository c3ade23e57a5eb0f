"""GPU path beyond the headline case, through the C ABI:

* the reference's free-hub diagnostic case (tests/test_validation.cpp:830-1022): the blade_sector
  fixture without the hub constraint, titanium, min_frequency 1 Hz, at 0 and 20000 rpm, both
  precisions, against the oracle: frequencies within 1e-6 relative, MAC >= 0.999.  Without the
  hub constraint K - M is indefinite, so the mixed path refines with restarted GMRES
  preconditioned by the FP32 factor (a problem whose refinement stalls is solved again in FP64);
* solve_parametric on the device equals solve_at_rpm per condition (src/cyclic_solver.cpp:1375-1485);
* the shift option: sigma = 0 gives the frequencies of the reference's sigma = 1 within 1e-8.
"""

import numpy as np
import pytest

from conftest import load_fixture

pytestmark = pytest.mark.gpu

FREQ_TOL = 1e-6
MAC_MIN = 0.999


def subspace_mac(phi, Psi):
    Q, _ = np.linalg.qr(Psi)
    v = Q.conj().T @ phi
    return float(np.real(np.vdot(v, v)) / np.real(np.vdot(phi, phi)))


@pytest.fixture(scope="module")
def blade():
    return load_fixture("blade_sector", 24)


@pytest.mark.parametrize("rpm", [0.0, 20000.0])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_free_hub_blade_sector_matches_oracle(oracle, blade, rpm, precision):
    from turbomodal_gb300.meshgen import Material
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    mat = Material(115e9, 0.33, 4430.0)
    s = CyclicSymmetrySolver(blade, mat, apply_hub_constraint=False, precision=precision)
    res = {r.harmonic_index: r for r in s.solve_at_rpm(rpm, 5, min_frequency=1.0)}
    om = oracle.OracleModel(blade, mat, apply_hub=False)
    om.prepare(rpm)
    ref = {r["harmonic_index"]: r for r in om.solve(rpm, 5, min_frequency=1.0, max_threads=8)}
    assert sorted(res) == sorted(ref)
    for k, o in ref.items():
        r = res[k]
        assert r.converged == o["converged"]
        assert len(r.frequencies) == len(o["frequencies"]), k
        err = np.abs(r.frequencies - o["frequencies"]) / o["frequencies"]
        assert err.max() <= FREQ_TOL, (k, err.max())
        for q in range(len(r.frequencies)):
            cluster = np.abs(o["frequencies"] - r.frequencies[q]) <= 1e-6 * r.frequencies[q]
            assert subspace_mac(r.mode_shapes[:, q], o["mode_shapes"][:, cluster]) >= MAC_MIN


def test_solve_parametric_on_device(cfg0_mesh):
    from turbomodal_gb300.meshgen import TITANIUM
    from turbomodal_gb300.solver import CyclicSymmetrySolver, ParametricCondition

    s = CyclicSymmetrySolver(cfg0_mesh, TITANIUM, precision="mixed")
    conds = [ParametricCondition(4000.0, 500.0), ParametricCondition(0.0, 300.0, [0.02, -0.01])]
    out = s.solve_parametric(conds, 4, [0, 3])
    assert len(out) == 2
    for cond, res in zip(conds, out):
        ref = s.solve_at_rpm(cond.rpm, 4, [0, 3])
        assert [r.harmonic_index for r in res] == [r.harmonic_index for r in ref] == [0, 3]
        for a, b in zip(res, ref):
            np.testing.assert_allclose(a.frequencies, b.frequencies, rtol=1e-12)


def test_shift_zero_gives_the_reference_shift_frequencies(cfg0_mesh):
    from turbomodal_gb300.meshgen import TITANIUM
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    s = CyclicSymmetrySolver(cfg0_mesh, TITANIUM, precision="fp64")
    assert s.get_option("shift") == 1.0
    a = {r.harmonic_index: r for r in s.solve_at_rpm(6000.0, 5, [0, 1, 18])}
    b = {r.harmonic_index: r for r in s.solve_at_rpm(6000.0, 5, [0, 1, 18], shift=0.0)}
    assert s.get_option("shift") == 1.0   # restored after the call
    for k in (0, 1, 18):
        np.testing.assert_allclose(b[k].frequencies, a[k].frequencies, rtol=1e-8)


def test_device_modal_mass_matches_host_formula(cfg0_mesh, oracle):
    """modal_mass_kg from the device (tmg_result_modal_mass) against the reference's host formula
    N Re(phi^H M phi) (python/turbomodal/solver.py:91-103) on the oracle's sector M: within 1e-12."""
    from turbomodal_gb300.meshgen import TITANIUM
    from turbomodal_gb300.solver import CyclicSymmetrySolver, _modal_mass_from_M, solve

    s = CyclicSymmetrySolver(cfg0_mesh, TITANIUM, precision="mixed")
    res = s.solve_at_rpm(7000.0, 6, [0, 2, 18])
    om = oracle.OracleModel(cfg0_mesh, TITANIUM)
    om.prepare(0.0)
    M = om.matrix("M")
    for r, host in zip(res, _modal_mass_from_M(M, res, cfg0_mesh.num_sectors)):
        assert r.modal_mass_kg.shape == host.shape and np.all(host > 0)
        np.testing.assert_allclose(r.modal_mass_kg, host, rtol=1e-12)
    enriched = solve(cfg0_mesh, TITANIUM, 7000.0, 6, harmonic_indices=[2], verbose=0, precision="mixed", solver=s)
    np.testing.assert_allclose(enriched[0].modal_mass_kg, res[1].modal_mass_kg, rtol=1e-9)


def test_interior_shift_mixed_refinement_converges(cfg0_mesh):
    """A shift inside the spectrum (sigma = (2 pi 600 Hz)^2, several modes below it) makes K - sigma M
    indefinite: the mixed path refines with restarted GMRES preconditioned by the FP32 factor.
    Its frequencies equal the FP64 path's within 1e-6, every refined solve ends within 10x of its
    1e-10 target (above 100x the problem would be solved again in FP64) and no problem falls back
    to FP64."""
    from turbomodal_gb300.meshgen import TITANIUM
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    sigma = (2 * np.pi * 600.0) ** 2
    mixed = CyclicSymmetrySolver(cfg0_mesh, TITANIUM, precision="mixed")
    a = {r.harmonic_index: r for r in mixed.solve_at_rpm(8000.0, 6, [0, 1, 7, 18], shift=sigma)}
    t = mixed.last_timing()
    assert t["retried_fp64"] == 0, t
    fp = CyclicSymmetrySolver(cfg0_mesh, TITANIUM, precision="fp64")
    b = {r.harmonic_index: r for r in fp.solve_at_rpm(8000.0, 6, [0, 1, 7, 18], shift=sigma)}
    assert sorted(a) == sorted(b) == [0, 1, 7, 18]
    for k in a:
        assert a[k].refine_residual <= 1e-9
        assert len(a[k].frequencies) == len(b[k].frequencies)
        assert np.max(np.abs(a[k].frequencies - b[k].frequencies) / b[k].frequencies) <= FREQ_TOL
