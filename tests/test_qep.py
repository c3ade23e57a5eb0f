"""Coriolis QEP, the Lancaster linearisation of src/modal_solver.cpp:151-312, on the host.

* Block layout: the library's lancaster_blocks (turbomodal_gb300/csrc/sym.cpp, run by
  tests/native/lancaster_check.cpp) against scipy.sparse.bmat on random patterns, with the device
  value formula of k_form_lancaster (turbomodal_gb300/csrc/engine.cu) restated in numpy.
* Oracle pins:
  - dense path (2n <= 200, the reference's wedge fixture): against scipy.linalg.eigh of the same
    pencil, with the reference's forward / backward selection;
  - Lanczos path: the reference's algorithm does not converge in its 20 restarts at its own shift
    sqrt(|K_k|_F / |M_k|_F).  The Ritz values it returns move by orders of magnitude under a
    1e-14 relative change of the input, so the GPU parity test of that path checks the result
    structure, not the values.
"""

import dataclasses
import os
import subprocess

import numpy as np
import pytest
import scipy.linalg as sl
import scipy.sparse as sp

from conftest import ROOT, load_fixture

CSRC = os.path.join(ROOT, "turbomodal_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    d = tmp_path_factory.mktemp("lanc")
    exe = str(d / "lancaster_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, os.path.join(ROOT, "tests", "native", "lancaster_check.cpp"),
                    os.path.join(CSRC, "sym.cpp"), "-o", exe], check=True)
    return exe, d


def rand_pattern(rng, n, density, diag=True):
    A = sp.random(n, n, density=density, random_state=rng, format="csc")
    A = sp.csc_matrix(A + A.T + (sp.eye(n) if diag else 0 * sp.eye(n)))
    A.data[:] = 1.0
    A.eliminate_zeros()
    A.sort_indices()
    return A


def run_blocks(checker, K, M, G):
    exe, d = checker
    src, dst = str(d / "in.bin"), str(d / "out.bin")
    with open(src, "wb") as f:
        np.array([K.shape[0]], np.int64).tofile(f)
        for P in (K, M, G):
            np.array([P.nnz], np.int64).tofile(f)
            P.indptr.astype(np.int64).tofile(f)
            P.indices.astype(np.int32).tofile(f)
    subprocess.run([exe, src, dst], check=True)
    raw = open(dst, "rb").read()
    n2 = 2 * K.shape[0]
    out, off = [], 0
    for _ in range(2):
        nnz = int(np.frombuffer(raw, np.int64, 1, off)[0]); off += 8
        p = np.frombuffer(raw, np.int64, n2 + 1, off); off += 8 * (n2 + 1)
        i = np.frombuffer(raw, np.int32, nnz, off); off += 4 * nnz
        srcs = []
        for _ in range(3):
            srcs.append(np.frombuffer(raw, np.int64, nnz, off)); off += 8 * nnz
        blk = np.frombuffer(raw, np.int8, nnz, off); off += nnz
        out.append(dict(p=p, i=i, sk=srcs[0], sm=srcs[1], sg=srcs[2], blk=blk))
    return out


def entry_cols(P):
    return np.repeat(np.arange(P.shape[1]), np.diff(P.indptr))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_lancaster_blocks_pattern_and_values(checker, seed):
    rng = np.random.default_rng(seed)
    n = 37
    K = rand_pattern(rng, n, 0.12)
    M = rand_pattern(rng, n, 0.05)
    G = rand_pattern(rng, n, 0.06, diag=False)
    A, L2 = run_blocks(checker, K, M, G)
    one = lambda P: sp.csc_matrix((np.ones(P.nnz), P.indices, P.indptr), shape=P.shape)
    refA = sp.csc_matrix(sp.bmat([[one(M) + one(G), one(K)], [one(K), one(K)]]))
    refL2 = sp.csc_matrix(sp.bmat([[one(M), None], [None, one(K)]]))
    for got, ref in ((A, refA), (L2, refL2)):
        ref.sort_indices()
        assert np.array_equal(got["p"], ref.indptr) and np.array_equal(got["i"], ref.indices)
    # every source index points at the entry of the same (row, col) in its block
    kc, mc, gc = entry_cols(K), entry_cols(M), entry_cols(G)
    for got, ref in ((A, refA), (L2, refL2)):
        rows = got["i"].astype(np.int64)
        cols = entry_cols(ref)
        blk = (rows >= n).astype(int) * 2 + (cols >= n).astype(int)   # 0 TL, 1 TR, 2 BL, 3 BR
        assert np.array_equal(got["blk"], np.array([0, 1, 2, 3])[blk])
        hk = got["sk"] >= 0
        assert np.array_equal(hk, blk > 0)
        assert np.array_equal(K.indices[got["sk"][hk]], rows[hk] % n)
        assert np.array_equal(kc[got["sk"][hk]], cols[hk] % n)
        for s, P, pc in (("sm", M, mc), ("sg", G, gc)):
            h = got[s] >= 0
            assert np.all(blk[h] == 0)
            assert np.array_equal(P.indices[got[s][h]], rows[h])
            assert np.array_equal(pc[got[s][h]], cols[h])
    # device value formula on random complex values
    Kv = rng.standard_normal(K.nnz) + 1j * rng.standard_normal(K.nnz)
    Mv = rng.standard_normal(M.nnz) + 1j * rng.standard_normal(M.nnz)
    Gv = rng.standard_normal(G.nnz) + 1j * rng.standard_normal(G.nnz)
    two_omega, sigma = 2093.4, 3.7e5
    Km = sp.csc_matrix((Kv, K.indices, K.indptr), shape=K.shape)
    Mm = sp.csc_matrix((Mv, M.indices, M.indptr), shape=M.shape)
    Gm = sp.csc_matrix((Gv, G.indices, G.indptr), shape=G.shape)
    L1d = sp.bmat([[1j * two_omega * Gm, Km], [Km, None]]).toarray()
    L2d = sp.bmat([[Mm, None], [None, Km]]).toarray()

    def form(g, mode):
        b = g["blk"]
        kv = np.where(g["sk"] >= 0, Kv[np.maximum(g["sk"], 0)], 0)
        gv = np.where(g["sg"] >= 0, (1j * two_omega) * Gv[np.maximum(g["sg"], 0)], 0)
        mv = np.where(g["sm"] >= 0, Mv[np.maximum(g["sm"], 0)], 0)
        l1 = np.where(b == 0, gv, np.where(b == 3, 0, kv))
        l2 = np.where(b == 0, mv, np.where(b == 3, kv, 0))
        v = l1 if mode == 1 else (l2 if mode == 2 else l1 - sigma * l2)
        return sp.csc_matrix((v, g["i"], g["p"]), shape=(2 * n, 2 * n)).toarray()

    assert np.allclose(form(A, 1), L1d, rtol=1e-15, atol=0)
    assert np.allclose(form(A, 2), L2d, rtol=1e-15, atol=0)
    assert np.allclose(form(A, 0), L1d - sigma * L2d, rtol=1e-15, atol=0)
    assert np.allclose(form(L2, 2), L2d, rtol=1e-15, atol=0)


def reference_selection(w, num_modes):
    """Forward / backward selection of src/modal_solver.cpp:249-296 on Lancaster eigenvalues w."""
    ent = sorted([x for x in w if abs(x) >= 1e-6], key=abs)
    fw = bw = 0
    sel = []
    for x in ent:
        if x > 0 and fw < num_modes:
            sel.append(x); fw += 1
        elif x < 0 and bw < num_modes:
            sel.append(x); bw += 1
        if fw >= num_modes and bw >= num_modes:
            break
    sel = sorted(sel, key=abs)[:num_modes]
    return np.abs(sel) / (2 * np.pi), np.where(np.array(sel) > 0, 1, -1)


def lancaster_eigs(om, k, omega):
    """Eigenvalues of the Hermitian parts of (L1, L2), as the reference's dense solver takes them
    (src/hermitian_lanczos.cpp:80-81).  The reference's G_k = Gc + P Gp + conj(P) Gp^H
    (src/cyclic_solver.cpp:987) is the Hermitian-sum formula of K_k applied to the skew gyroscopic
    matrix, so D = i 2 omega G_k is not Hermitian (|D - D^H| / |D| is about 0.67 here) and the
    symmetrisation changes L1."""
    K = om.matrix("Kk", k=k).toarray()
    M = om.matrix("Mk", k=k).toarray()
    G = om.matrix("Gk", k=k).toarray()
    Z = np.zeros_like(K)
    L1 = np.block([[2j * omega * G, K], [K, Z]])
    L2 = np.block([[M, Z], [Z, K]])
    return sl.eigh(0.5 * (L1 + L1.conj().T), 0.5 * (L2 + L2.conj().T), eigvals_only=True)


def test_oracle_qep_dense_path_against_scipy(oracle):
    """2n <= 200: the oracle's dense QEP equals scipy's eigenvalues of the Lancaster pencil,
    with forward and backward whirl split around the rotating-frame frequency."""
    from turbomodal_gb300.meshgen import STEEL

    m = load_fixture("wedge_sector", 24)
    rpm = 10000.0
    omega = rpm * 2 * np.pi / 60
    om = oracle.OracleModel(m, STEEL)
    om.prepare(rpm, True)
    assert 2 * len(om.free_map()) <= 200
    res = {r["harmonic_index"]: r for r in om.solve(rpm, 5, harmonic_indices=[1, 2, 12], max_threads=4,
                                                  include_coriolis=True)}
    for k in (1, 2, 12):
        f_ref, w_ref = reference_selection(lancaster_eigs(om, k, omega), 5)
        r = res[k]
        assert r["converged"]
        assert np.max(np.abs(r["frequencies"] - f_ref) / f_ref) < 1e-8
        if k == 12:   # k = N/2: real operators, exact +/- pairs; which sign comes first is a tie
            f, w = r["frequencies"], r["whirl_direction"]
            for i in range(0, len(f) - 1, 2):
                assert abs(f[i] - f[i + 1]) <= 1e-9 * f[i] and w[i] == -w[i + 1]
        else:
            assert np.array_equal(r["whirl_direction"], w_ref)
    std = {r["harmonic_index"]: r for r in om.solve(rpm, 5, harmonic_indices=[1], max_threads=4)}
    f_std = std[1]["frequencies"][0]
    f_fw = res[1]["frequencies"][res[1]["whirl_direction"] == 1][0]
    f_bw = res[1]["frequencies"][res[1]["whirl_direction"] == -1][0]
    assert min(f_fw, f_bw) < f_std * (1 + 1e-3) and max(f_fw, f_bw) > f_std * (1 - 1e-3)


def test_oracle_qep_lanczos_path_is_unconverged_and_input_sensitive(oracle):
    """2n > 200 at the reference's shift: 20 restarts without convergence, and a 1e-14 relative
    change of Young's modulus changes the returned frequencies by more than 1e-3 relative."""
    from turbomodal_gb300.meshgen import TITANIUM, sector_mesh

    m = sector_mesh(4, 3, 1, num_sectors=24, jitter=0.02, seed=3)
    rpm = 10000.0
    out = []
    for mat in (TITANIUM, dataclasses.replace(TITANIUM, E=TITANIUM.E * (1 + 1e-14))):
        om = oracle.OracleModel(m, mat)
        res = om.solve(rpm, 5, harmonic_indices=[1], max_threads=4, include_coriolis=True)
        assert len(res) == 1
        r = res[0]
        assert not r["converged"] and r["iterations"] == 20
        assert set(np.unique(r["whirl_direction"])) <= {-1, 1}
        out.append(r["frequencies"])
    n = min(len(out[0]), len(out[1]))
    assert n > 0
    assert np.max(np.abs(out[0][:n] - out[1][:n]) / out[0][:n]) > 1e-3
