"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle.

Tolerances (written here, from the target): CSC pattern, AMD order, elimination tree and
column counts bit-exact; element-derived matrices bit-exact (same arithmetic, no FMA);
matrices that pass through the static prestress solve within 1e-12 relative; frequencies
within 1e-6 relative of the FP64 oracle; mode MAC >= 0.999.
"""

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import load_fixture

pytestmark = pytest.mark.gpu

FREQ_TOL = 1e-6
MAC_MIN = 0.999
ROT_TOL = 1e-12


@pytest.fixture(scope="module")
def cfg0():
    from turbomodal_gb300.meshgen import config_mesh

    return config_mesh(0)


@pytest.fixture(scope="module")
def gpu_solvers(cfg0):
    from turbomodal_gb300.meshgen import STEEL, TITANIUM
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    return {0.0: CyclicSymmetrySolver(cfg0, STEEL), 10000.0: CyclicSymmetrySolver(cfg0, TITANIUM)}


@pytest.fixture(scope="module")
def oracles(cfg0, oracle):
    from turbomodal_gb300.meshgen import STEEL, TITANIUM

    out = {}
    for rpm, mat in ((0.0, STEEL), (10000.0, TITANIUM)):
        om = oracle.OracleModel(cfg0, mat)
        om.prepare(rpm)
        out[rpm] = om
    return out


@pytest.fixture(scope="module")
def oracle_results(oracles):
    return {rpm: {r["harmonic_index"]: r for r in om.solve(rpm, 5, max_threads=8)} for rpm, om in oracles.items()}


def same_pattern(A, B):
    A = sp.csc_matrix(A); B = sp.csc_matrix(B)
    A.sort_indices(); B.sort_indices()
    return A.shape == B.shape and np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)


def rel_diff(A, B):
    d = abs(sp.csc_matrix(A) - sp.csc_matrix(B)).max()
    return d / max(abs(sp.csc_matrix(B)).max(), 1e-300)


@pytest.mark.parametrize("name", ["K", "M"])
def test_sector_assembly_bit_exact(gpu_solvers, oracles, name):
    G = gpu_solvers[0.0].assemble(name)
    O = oracles[0.0].matrix(name)
    assert same_pattern(G, O)
    assert np.array_equal(G.data, O.data)


def test_rotating_element_assembly_bit_exact(gpu_solvers, cfg0, oracle):
    from turbomodal_gb300.meshgen import TITANIUM

    s = gpu_solvers[10000.0]
    om = oracle.OracleModel(cfg0, TITANIUM)
    omega = 10000.0 * 2 * np.pi / 60
    for name in ("Komega", "G"):
        G = s.assemble(name, 10000.0)
        O = om.matrix(name, param=omega)
        assert same_pattern(G, O)
        assert np.array_equal(G.data, O.data)


def test_prestress_and_effective_stiffness(gpu_solvers, oracles):
    s = gpu_solvers[10000.0]
    for name in ("Ksigma", "Keff"):
        G = s.assemble(name, 10000.0)
        O = oracles[10000.0].matrix(name)
        assert same_pattern(G, O)
        assert rel_diff(G, O) <= ROT_TOL


@pytest.mark.parametrize("name", ["Kcf", "Kpf", "Mcf", "Mpf", "K0r", "M0r", "Khr", "Mhr"])
def test_projections_bit_exact_at_rest(gpu_solvers, oracles, name):
    s = gpu_solvers[0.0]
    s.prepare(0.0)
    G = s.projection(name)
    O = oracles[0.0].matrix(name)
    assert same_pattern(G, O)
    assert np.array_equal(np.asarray(G.data), np.asarray(O.data))


@pytest.mark.parametrize("name", ["Kcf", "Kpf", "Mcf", "Mpf", "K0r", "M0r"])
def test_projections_rotating(gpu_solvers, oracles, name):
    """At speed, the projected stiffness inherits the prestress solve's last-bit differences.
    Entries whose exact value is zero survive the reference's pruning (|v| <= 1e-27) only as
    roundoff; such entries may appear on one side only.  Every other entry matches within 1e-12."""
    s = gpu_solvers[10000.0]
    s.prepare(10000.0)
    G = sp.csc_matrix(s.projection(name))
    O = sp.csc_matrix(oracles[10000.0].matrix(name))
    scale = abs(O).max()
    D = (G - O).tocsc()
    assert abs(D).max() <= ROT_TOL * scale
    onlyG = abs(G).multiply(abs(O) == 0)
    onlyO = abs(O).multiply(abs(G) == 0)
    for X in (onlyG, onlyO):
        if X.nnz:
            assert abs(X).max() <= 1e-14 * scale
    assert (G != 0).sum() - (O != 0).sum() in range(-50, 51)


@pytest.mark.parametrize("kind,k", [(0, 1), (1, 0), (2, 18)])
def test_symbolic_bit_exact(gpu_solvers, oracles, oracle, kind, k):
    """AMD order, elimination tree and column counts of K_k - sigma M_k equal the oracle's
    restatement of SimplicialLDLT::analyzePattern (hermitian_lanczos.cpp:20)."""
    s = gpu_solvers[0.0]
    s.prepare(0.0)
    perm, parent, cc = s.symbolic(kind)
    om = oracles[0.0]
    if kind == 0:
        Kk, Mk = om.matrix("Kk", k=k), om.matrix("Mk", k=k)
    else:
        Kk, Mk = om.matrix("K0r" if kind == 1 else "Khr"), om.matrix("M0r" if kind == 1 else "Mhr")
    P = sp.tril(sp.csc_matrix((abs(Kk) + abs(Mk)) > 0, dtype=float)).tocsc()
    op, opar, occ = oracle.ldl_symbolic(P)
    assert np.array_equal(perm, op)
    assert np.array_equal(parent, opar)
    assert np.array_equal(cc, occ)


def subspace_mac(phi, Psi):
    """Largest MAC of phi against the span of the columns of Psi."""
    Q, _ = np.linalg.qr(Psi)
    v = Q.conj().T @ phi
    return float(np.real(np.vdot(v, v)) / np.real(np.vdot(phi, phi)))


def check_against_oracle(res, ref):
    assert sorted(r.harmonic_index for r in res) == sorted(ref)
    for r in res:
        o = ref[r.harmonic_index]
        assert r.converged
        assert len(r.frequencies) == len(o["frequencies"])
        err = np.abs(r.frequencies - o["frequencies"]) / o["frequencies"]
        assert err.max() <= FREQ_TOL, (r.harmonic_index, err.max())
        assert np.array_equal(r.whirl_direction, o["whirl_direction"])
        for m in range(len(r.frequencies)):
            f = r.frequencies[m]
            cluster = np.abs(o["frequencies"] - f) <= 1e-6 * f
            # degenerate pairs (x, conj x) and near-coincident modes: subspace MAC
            assert subspace_mac(r.mode_shapes[:, m], o["mode_shapes"][:, cluster]) >= MAC_MIN


@pytest.mark.parametrize("rpm", [0.0, 10000.0])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_frequencies_and_modes_match_oracle(gpu_solvers, oracle_results, rpm, precision):
    res = gpu_solvers[rpm].solve_at_rpm(rpm, 5, precision=precision)
    check_against_oracle(res, oracle_results[rpm])


def test_batch_same_alone_and_in_the_mix(gpu_solvers):
    """A harmonic solved alone gives the result it gives inside the full batch."""
    s = gpu_solvers[10000.0]
    full = {r.harmonic_index: r for r in s.solve_at_rpm(10000.0, 5, precision="mixed")}
    for k in (3, 11):
        alone = s.solve_at_rpm(10000.0, 5, harmonic_indices=[k], precision="mixed")[0]
        np.testing.assert_allclose(alone.frequencies, full[k].frequencies, rtol=1e-9)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_speed_sequence_same_as_fresh(cfg0, precision):
    """A solver that has already solved at rest (a different sparsity pattern, so the symbolic
    analysis is redone) gives the result a fresh solver gives at speed."""
    from turbomodal_gb300.meshgen import TITANIUM
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    s = CyclicSymmetrySolver(cfg0, TITANIUM)
    s.solve_at_rpm(0.0, 5, precision=precision)
    s.solve_at_rpm(5000.0, 5, precision=precision)
    seq = {r.harmonic_index: r for r in s.solve_at_rpm(10000.0, 5, precision=precision)}
    fresh = {r.harmonic_index: r for r in CyclicSymmetrySolver(cfg0, TITANIUM).solve_at_rpm(10000.0, 5,
                                                                                             precision=precision)}
    assert sorted(seq) == sorted(fresh)
    for k in fresh:
        np.testing.assert_allclose(seq[k].frequencies, fresh[k].frequencies, rtol=1e-9)


@pytest.mark.parametrize("rpm", [0.0, 6000.0])
def test_dense_path_small_sector(oracle, rpm):
    """n <= 200 (the reference's wedge fixture, 66 free DOF per harmonic): the dense generalized
    eigensolver against the oracle's restatement of solve_dense (hermitian_lanczos.cpp:68-110)."""
    from turbomodal_gb300.meshgen import STEEL
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    m = load_fixture("wedge_sector", 24)
    res = CyclicSymmetrySolver(m, STEEL).solve_at_rpm(rpm, 5)
    om = oracle.OracleModel(m, STEEL)
    om.prepare(rpm)
    ref = {r["harmonic_index"]: r for r in om.solve(rpm, 5)}
    check_against_oracle(res, ref)


def test_leissa_clamped_disk_gpu(oracle):
    from turbomodal_gb300.meshgen import Material
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    m = load_fixture("leissa_disk_sector", 24)
    E, nu, rho, h, a = 200e9, 0.33, 7850.0, 0.01, 0.3
    s = CyclicSymmetrySolver(m, Material(E, nu, rho))
    res = {r.harmonic_index: r for r in s.solve_at_rpm(0.0, 5, harmonic_indices=[0, 1, 2, 3])}
    D = E * h ** 3 / (12 * (1 - nu ** 2))
    for nd, lam2 in enumerate([4.235, 3.482, 5.499, 12.23]):
        fa = lam2 / (2 * np.pi * a * a) * np.sqrt(D / (rho * h))
        assert abs(res[nd].frequencies[0] - fa) / fa < (0.15 if nd == 3 else 0.10)
    om = oracle.OracleModel(m, Material(E, nu, rho))
    om.prepare(0.0)
    ref = {r["harmonic_index"]: r for r in om.solve(0.0, 5, harmonic_indices=[0, 1, 2, 3], with_shapes=False)}
    for k, r in res.items():
        assert np.max(np.abs(r.frequencies - ref[k]["frequencies"]) / ref[k]["frequencies"]) <= FREQ_TOL


def test_full_size_sector_properties():
    """Config-1 mesh (57,897 nodes) at one speed: mixed vs FP64 frequencies within 1e-6 and
    mode MAC >= 0.999, ascending frequencies, bounded residuals, every refined solve at its
    1e-10 target, finite positive modal masses (size-independent properties)."""
    from turbomodal_gb300.meshgen import TITANIUM, config_mesh
    from turbomodal_gb300.solver import CyclicSymmetrySolver, _modal_mass_from_M

    m = config_mesh(1)
    s = CyclicSymmetrySolver(m, TITANIUM)
    ks = [0, 1, 9, 18]
    mixed = s.solve_at_rpm(8000.0, 10, harmonic_indices=ks, precision="mixed")
    fp64 = s.solve_at_rpm(8000.0, 10, harmonic_indices=ks, precision="fp64")
    for a, b in zip(mixed, fp64):
        assert a.harmonic_index == b.harmonic_index
        assert np.all(np.diff(b.frequencies) >= -1e-9 * b.frequencies[1:])
        assert np.max(np.abs(a.frequencies - b.frequencies) / b.frequencies) <= FREQ_TOL
        assert b.max_residual < 1e-6 and a.max_residual < 1e-3
        assert a.refine_residual <= 1e-10
        for q in range(len(a.frequencies)):
            cluster = np.abs(b.frequencies - a.frequencies[q]) <= 1e-6 * a.frequencies[q]
            assert subspace_mac(a.mode_shapes[:, q], b.mode_shapes[:, cluster]) >= MAC_MIN
    M = s.assemble("M")
    for mm in _modal_mass_from_M(M, fp64, m.num_sectors):
        assert np.all(np.isfinite(mm)) and np.all(mm > 0)


def test_errors_are_reported(cfg0):
    from turbomodal_gb300.meshgen import STEEL
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    s = CyclicSymmetrySolver(cfg0, STEEL)
    with pytest.raises(ValueError):
        s.solve_at_rpm(0.0, 0)
    bad = type(cfg0)()
    bad.nodes = cfg0.nodes
    bad.elements = cfg0.elements.copy()
    bad.elements[0, 0] = cfg0.num_nodes() + 5
    bad.node_sets = cfg0.node_sets
    bad.left_boundary, bad.right_boundary, bad.matched_pairs = cfg0.left_boundary, cfg0.right_boundary, cfg0.matched_pairs
    bad.num_sectors = cfg0.num_sectors
    with pytest.raises(ValueError):
        CyclicSymmetrySolver(bad, STEEL)


def test_smoke_entry():
    import __graft_entry__ as g

    g.smoke()
