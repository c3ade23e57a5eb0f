"""The reference's own rotating-frame and Coriolis test cases replayed on the oracle (CPU), with the
product's host-side result consumers (turbomodal_gb300.solver.compute_stationary_frame) where the
reference test uses them.

Sources: tests/test_cyclic.cpp:539-720 (Coriolis cases), tests/test_rotating.cpp (whirl labels,
rotating-frame frequencies, stationary-frame ordering) and tests/test_solver.cpp (M-orthogonality,
determinism), all on the reference's wedge fixture with E = 200 GPa, nu = 0.3, rho = 7850 kg/m^3
and 24 sectors.
"""

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import load_fixture

MAT = dict(E=200e9, nu=0.3, rho=7850.0)


@pytest.fixture(scope="module")
def wedge():
    return load_fixture("wedge_sector", 24)


@pytest.fixture(scope="module")
def model(oracle, wedge):
    from turbomodal_gb300.meshgen import Material

    return oracle.OracleModel(wedge, Material(**MAT))


def by_k(results):
    return {r["harmonic_index"]: r for r in results}


def test_whirl_labels_without_coriolis(model, wedge):
    """test_cyclic.cpp:539-563 (CoriolisOffMatchesBaseline), test_rotating.cpp FWBWSplittingAtNonzeroRPM
    and StandingWavesAtK0: standing harmonics (k = 0, N/2) carry whirl 0; the degenerate ones
    carry +1 / -1 pairs."""
    res = model.solve(5000.0, 5, max_threads=4)
    assert len(res) == wedge.num_sectors // 2 + 1
    for r in res:
        k = r["harmonic_index"]
        w = r["whirl_direction"]
        if k == 0 or 2 * k == wedge.num_sectors:
            assert np.all(w == 0)
        else:
            assert np.all(w != 0) and (w == 1).any() and (w == -1).any()


def test_coriolis_k0_uses_standard_path(model):
    """test_cyclic.cpp:565-577: k = 0 with Coriolis is solved by the standard path (whirl 0)."""
    r = model.solve(5000.0, 5, harmonic_indices=[0], max_threads=4, include_coriolis=True)
    assert len(r) == 1 and r[0]["harmonic_index"] == 0 and np.all(r[0]["whirl_direction"] == 0)


def test_coriolis_at_rest_is_no_coriolis(model):
    """test_cyclic.cpp:579-597: at 0 rpm the Coriolis flag changes nothing (1e-6 Hz)."""
    a = model.solve(0.0, 5, harmonic_indices=[3], max_threads=4)
    b = model.solve(0.0, 5, harmonic_indices=[3], max_threads=4, include_coriolis=True)
    n = min(len(a[0]["frequencies"]), len(b[0]["frequencies"]))
    assert n > 0
    assert np.max(np.abs(a[0]["frequencies"][:n] - b[0]["frequencies"][:n])) <= 1e-6


def test_coriolis_splits_forward_and_backward(model):
    """test_cyclic.cpp:599-642: at 10000 rpm with Coriolis, k = 3 has forward and backward modes and
    the first forward rotating-frame frequency exceeds the first backward one."""
    r = model.solve(10000.0, 10, harmonic_indices=[3], max_threads=4, include_coriolis=True)
    assert len(r) == 1 and r[0]["harmonic_index"] == 3
    w, f = r[0]["whirl_direction"], r[0]["frequencies"]
    assert (w == 1).any() and (w == -1).any()
    assert f[w == 1][0] > f[w == -1][0]


def test_gyroscopic_projection(oracle, wedge, model):
    """test_cyclic.cpp:678-720: G is skew-symmetric and its direct projection T(3)^H G T(3) is
    skew-Hermitian (1e-10 of its norm).  The solver's own G_k = Gc + P Gp + conj(P) Gp^H
    (src/cyclic_solver.cpp:987), which the reference's QEP uses, is not: the split sum takes the
    (right, non-right) block as the transpose of the (non-right, right) block, which holds for the
    symmetric K and M but flips sign for the skew G."""
    G = model.matrix("G")
    assert abs(G + G.T).max() <= 1e-10 * sp.linalg.norm(G)
    T = model.matrix("T", k=3)
    Gd = (T.conj().T @ G.astype(complex) @ T).tocsc()
    assert abs(Gd + Gd.conj().T).max() <= 1e-10 * sp.linalg.norm(Gd)
    model.prepare(10000.0, True)
    Gk = model.matrix("Gk", k=3)
    assert sp.linalg.norm(Gk + Gk.conj().T) > 0.1 * sp.linalg.norm(Gk)


def test_stationary_frame_forward_above_backward(model, wedge):
    """test_rotating.cpp FWGreaterThanBWInStationaryFrame: for every degenerate harmonic at 5000 rpm,
    the highest forward stationary-frame frequency exceeds the lowest backward one."""
    from turbomodal_gb300.solver import ModalResult, compute_stationary_frame

    for r in model.solve(5000.0, 3, max_threads=4):
        k = r["harmonic_index"]
        if not (0 < k < wedge.num_sectors // 2):
            continue
        mr = ModalResult(k, r["rpm"], r["frequencies"], r["mode_shapes"], r["whirl_direction"], r["converged"])
        sf = compute_stationary_frame(mr, wedge.num_sectors)
        fw = sf.frequencies[sf.whirl_direction == 1]
        bw = sf.frequencies[sf.whirl_direction == -1]
        if len(fw) and len(bw):
            assert fw.max() > bw.min()


def test_frequencies_change_with_speed(model):
    """test_rotating.cpp FrequenciesChangeWithRPM: k = 0 frequencies at 10000 rpm differ from 0 rpm."""
    a = by_k(model.solve(0.0, 3, harmonic_indices=[0], max_threads=4))[0]["frequencies"]
    b = by_k(model.solve(10000.0, 3, harmonic_indices=[0], max_threads=4))[0]["frequencies"]
    n = min(len(a), len(b))
    assert n >= 1
    assert np.max(np.abs(a[:n] - b[:n]) / a[:n]) > 1e-6


def hub_clamped(model, wedge):
    """The wedge's K and M with the hub nodes' DOFs removed (ModalSolver::eliminate_dofs,
    src/modal_solver.cpp:314-360), no cyclic constraint."""
    hub = wedge.find_node_set("hub_constraint").node_ids
    fixed = set(3 * n + c for n in hub for c in range(3))
    keep = np.array([d for d in range(wedge.num_dof()) if d not in fixed])
    K = model.matrix("K").tocsc()[keep][:, keep]
    M = model.matrix("M").tocsc()[keep][:, keep]
    return sp.csc_matrix(K), sp.csc_matrix(M)


def test_wedge_modes_m_orthogonal_and_deterministic(oracle, model, wedge):
    """tests/test_solver.cpp WedgeSectorMOrthogonality and SolverDeterministic: ten modes of the
    hub-clamped wedge are M-orthogonal (1e-6 of the geometric mean of their M-norms) and two solves
    give bit-identical eigenvalues (the reference allows 1e-15)."""
    K, M = hub_clamped(model, wedge)
    ev1, V, info = oracle.lanczos(K, M, 10, shift=1.0, maxit=1000)
    ev2, _, _ = oracle.lanczos(K, M, 10, shift=1.0, maxit=1000)
    assert info[1] == 1 and len(ev1) >= 5
    assert np.array_equal(ev1, ev2)
    G = V.conj().T @ (M @ V)
    d = np.real(np.diag(G))
    assert np.all(d > 0)
    off = np.abs(G - np.diag(np.diag(G)))
    assert np.all(off <= 1e-6 * np.sqrt(np.outer(d, d)))


def test_wedge_assembly_cases(oracle, wedge):
    """tests/test_assembler.cpp WedgeSectorDimensions, WedgeSectorMPositiveSemiDefinite,
    WedgeSectorKNonNegativeEigenvalues, KScalesWithE, MScalesWithRho, MIndependentOfE (on the wedge
    rather than one element)."""
    from turbomodal_gb300.meshgen import Material

    def km(E, rho):
        om = oracle.OracleModel(wedge, Material(E, 0.3, rho))
        return om.matrix("K").toarray(), om.matrix("M").toarray()

    K, M = km(200e9, 7850.0)
    ndof = wedge.num_dof()
    assert K.shape == (ndof, ndof) and M.shape == (ndof, ndof)
    em = np.linalg.eigvalsh(M)
    ek = np.linalg.eigvalsh(K)
    assert em.min() > -1e-10 * em.max()
    assert ek.min() > -1e-6 * ek.max()
    assert np.sum(np.abs(ek) <= 1e-9 * ek.max()) == 6       # six rigid-body modes of the free sector
    K2, M2 = km(400e9, 7850.0)
    assert np.allclose(K2, 2.0 * K, rtol=1e-10, atol=1e-10 * np.abs(K).max())
    assert np.array_equal(M2, M)
    _, M3 = km(200e9, 15700.0)
    assert np.allclose(M3, 2.0 * M, rtol=1e-10, atol=0)


@pytest.mark.parametrize("k", [1, 5, 12])
def test_split_projection_equals_direct_projection(oracle, wedge, k):
    """The solver's per-harmonic sums K_k = Kc + P Kp + conj(P) Kp^H and the same for M
    (src/cyclic_solver.cpp:560-671, :942-947) equal the direct projection T(k)^H A T(k) of the
    sector matrix, restricted to the free DOFs (1e-12 of the matrix scale), for the effective
    stiffness at 10000 rpm and for the mass."""
    from turbomodal_gb300.meshgen import Material

    om = oracle.OracleModel(wedge, Material(**MAT))
    om.prepare(10000.0)
    free = om.free_map()
    T = om.matrix("T", k=k).tocsc()
    for name, split in (("Keff", "Kk"), ("M", "Mk")):
        A = om.matrix(name).astype(complex)
        D = (T.conj().T @ A @ T).tocsc()[free][:, free].toarray()
        S = om.matrix(split, k=k).toarray()
        assert np.abs(D - S).max() <= 1e-12 * np.abs(D).max()


def test_static_prestress_solve_against_sparse_direct(oracle, wedge):
    """static_centrifugal (src/cyclic_solver.cpp:456-558): the prestress displacement solves the
    k = 0 cyclic system with the hub DOFs removed, (T0^T K T0)_free u_cyc = (T0^T F)_free, u = T0 u_cyc.
    Checked against scipy's sparse direct solve of the same system (1e-10 relative)."""
    import scipy.sparse.linalg as spla
    from turbomodal_gb300.meshgen import Material

    om = oracle.OracleModel(wedge, Material(**MAT))
    rpm = 10000.0
    om.prepare(rpm)
    omega = rpm * 2 * np.pi / 60
    T = om.matrix("T", k=0).tocsc().real
    K = om.matrix("K").tocsc()
    F = om.centrifugal(omega)
    free = om.free_map()
    Kc = (T.T @ K @ T).tocsc()[free][:, free]
    Fc = (T.T @ F)[free]
    uc = np.zeros(T.shape[1])
    uc[free] = spla.spsolve(Kc.tocsc(), Fc)
    u = T @ uc
    got = om.static_u()
    assert np.abs(got - u).max() <= 1e-10 * np.abs(u).max()
