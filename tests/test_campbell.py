"""Consumers of a result set (host side): stationary-frame conversion with the reference's own
test cases (tests/test_cyclic.cpp:451-535), Campbell arrays and the CSV exports."""

import numpy as np
import pytest

from turbomodal_gb300.solver import (ModalResult, campbell_data, compute_stationary_frame, export_campbell_csv,
                                     export_zzenf_csv)


def result(k, rpm, freqs, whirl=None):
    f = np.asarray(freqs, dtype=float)
    w = np.zeros(len(f), np.int32) if whirl is None else np.asarray(whirl, np.int32)
    return ModalResult(k, rpm, f, np.zeros((6, len(f)), np.complex128), w)


def test_fw_bw_split():
    sf = compute_stationary_frame(result(3, 6000.0, [500.0, 1000.0]), 24)
    np.testing.assert_allclose(sf.frequencies, [200.0, 700.0, 800.0, 1300.0], atol=0.1)
    assert sf.whirl_direction.tolist() == [-1, -1, 1, 1]


def test_no_split_at_k0_kN2_and_rest():
    for k, rpm in ((0, 6000.0), (12, 6000.0), (5, 0.0)):
        f = [100.0, 200.0, 300.0] if k == 0 else [500.0, 1000.0]
        sf = compute_stationary_frame(result(k, rpm, f), 24)
        np.testing.assert_allclose(sf.frequencies, f, atol=1e-10)
        assert not sf.whirl_direction.any()


def test_whirl_carrying_modes_move_per_mode():
    # degenerate pairs carry +1/-1: each mode moves by whirl * k * Omega / 2 pi (300 Hz here)
    sf = compute_stationary_frame(result(3, 6000.0, [500.0, 500.0], [1, -1]), 24)
    np.testing.assert_allclose(sf.frequencies, [200.0, 800.0])
    assert sf.whirl_direction.tolist() == [-1, 1]


def test_campbell_arrays():
    sweep = [[result(0, 0.0, [100.0, 200.0]), result(3, 0.0, [500.0])],
             [result(0, 6000.0, [110.0, 210.0]), result(3, 6000.0, [500.0])]]
    d = campbell_data(sweep, num_sectors=24)
    assert d["frequencies"].shape == (2, 2, 4)
    assert d["harmonic_index"].tolist() == [0, 3]
    np.testing.assert_allclose(d["rpm"], [0.0, 6000.0])
    np.testing.assert_allclose(d["frequencies"][1, 1, :2], [200.0, 800.0])
    assert d["whirl_direction"][1, 1, :2].tolist() == [-1, 1]
    np.testing.assert_allclose(d["frequencies"][1, 0, :2], [110.0, 210.0])
    assert np.isnan(d["frequencies"][0, 0, 2:]).all()


def test_csv_exports(tmp_path):
    rows = [[result(3, 6000.0, [500.0, 1000.0])]]
    p = tmp_path / "campbell.csv"
    export_campbell_csv(str(p), rows, 24)
    lines = p.read_text().splitlines()
    assert lines[0] == "rpm,harmonic_index,mode_family,frequency_hz,whirl_direction"
    assert lines[1] == "6000.000000,3,1,200.000000,-1"
    assert len(lines) == 5
    q = tmp_path / "zzenf.csv"
    export_zzenf_csv(str(q), rows[0])
    assert q.read_text().splitlines() == ["nodal_diameter,mode_family,frequency_hz,rpm", "3,1,500.000000,6000.000000",
                                          "3,2,1000.000000,6000.000000"]


def test_modal_mass_enrichment():
    """modal_mass_kg = N * Re(phi^H M_sector phi) per mode (python/turbomodal/solver.py:91-103)."""
    import scipy.sparse as sp

    from turbomodal_gb300.solver import EnrichedModalResult, _modal_mass_from_M

    rng = np.random.default_rng(0)
    A = rng.standard_normal((6, 6))
    M = sp.csc_matrix(A @ A.T + 6 * np.eye(6))
    phi = rng.standard_normal((6, 2)) + 1j * rng.standard_normal((6, 2))
    r = ModalResult(1, 0.0, np.array([1.0, 2.0]), phi, np.zeros(2, np.int32))
    (mm,) = _modal_mass_from_M(M, [r], 24)
    expect = [24 * np.real(np.vdot(phi[:, q], M @ phi[:, q])) for q in range(2)]
    np.testing.assert_allclose(mm, expect, rtol=1e-13)
    e = EnrichedModalResult(_result=r, modal_mass_kg=mm)
    assert e.harmonic_index == 1 and e.modal_mass_kg is mm


def test_solve_parametric_is_solve_at_rpm_per_condition():
    """src/cyclic_solver.cpp:1375-1485: the reference's per-condition K_eff is overwritten by the
    solve_at_rpm it calls (:737-820), so each condition returns solve_at_rpm(condition.rpm) with
    the call's other arguments; progress is reported once per condition."""
    from turbomodal_gb300.solver import CyclicSymmetrySolver, ParametricCondition

    calls, prog = [], []
    s = CyclicSymmetrySolver.__new__(CyclicSymmetrySolver)
    s.solve_at_rpm = lambda *a: calls.append(a) or [a[0]]
    conds = [ParametricCondition(3000.0, 400.0), ParametricCondition(0.0), ParametricCondition(9000.0, 900.0, [0.01])]
    out = s.solve_parametric(conds, 7, [1, 2], 3, True, 5.0, progress_cb=prog.append)
    assert out == [[3000.0], [0.0], [9000.0]]
    assert [c[:6] for c in calls] == [(r, 7, [1, 2], 3, True, 5.0) for r in (3000.0, 0.0, 9000.0)]
    assert [p.completed for p in prog] == [1, 2, 3] and all(p.harmonic_k == -1 and p.total == 3 for p in prog)


def test_module_functions_take_the_reference_parameters():
    """tm.solve and tm.rpm_sweep keep the reference's parameter names, order and defaults
    (python/turbomodal/solver.py:237-255 and :499-514), so positional calls mean the same; the
    GPU path's own options are keyword-only at the end."""
    import inspect

    from turbomodal_gb300 import solver as m

    solve_ref = [("mesh", None), ("material", None), ("rpm", 0.0), ("num_modes", 20), ("fluid", None),
                 ("config", None), ("verbose", m.PROGRESS), ("harmonic_indices", None), ("max_threads", 0),
                 ("hub_constraint", "fixed"), ("include_coriolis", False), ("min_frequency", 0.0),
                 ("temperature", None), ("condition", None), ("boundary_conditions", None),
                 ("show_convergence", False), ("memory_reserve_fraction", 0.2)]
    sweep_ref = [("mesh", None), ("material", None), ("rpm_values", None), ("num_modes", 20), ("fluid", None),
                 ("verbose", m.SILENT), ("harmonic_indices", None), ("max_threads", 0), ("hub_constraint", "fixed"),
                 ("include_coriolis", False), ("min_frequency", 0.0), ("temperature", None),
                 ("boundary_conditions", None), ("memory_reserve_fraction", 0.2)]
    for fn, ref in ((m.solve, solve_ref), (m.rpm_sweep, sweep_ref)):
        ps = [p for p in inspect.signature(fn).parameters.values() if p.kind != p.KEYWORD_ONLY]
        assert [p.name for p in ps] == [n for n, _ in ref]
        for p, (_, d) in zip(ps, ref):
            if d is not None or p.default is not inspect.Parameter.empty:
                assert p.default == d, p.name
    assert (m.SILENT, m.PROGRESS, m.DETAILED) == (0, 1, 2)


def test_solve_rejects_constraint_groups():
    from turbomodal_gb300.solver import solve

    with pytest.raises(NotImplementedError):
        solve(None, None, boundary_conditions=[object()], verbose=0)
