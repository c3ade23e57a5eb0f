"""The deflated refinement CG of the mixed-precision shift-invert apply, restated on the CPU.

The sequence is that of ShiftInvertB::apply with set_deflation (turbomodal_gb300/csrc/engine.cu),
which the solver enables with TMG_DEFLATE:
- x0 = W E^-1 W^H b with E = W^H A W;
- z = F^-1 r, then z -= W E^-1 (A W)^H z after every preconditioner solve;
- CG in FP64 on A = K_k - M_k, preconditioned by an FP32 factor F of the Jacobi-scaled operator.
W holds the lowest eigenvectors of the same harmonic at another speed.  Checked here: both
iterations stop at the product's target (recursive residual 1e-10; the true residual within 10x
of it, the usual CG residual gap) with the direct solution, and the deflated one in fewer
preconditioner solves.
"""

import numpy as np
import scipy.linalg as sl


def pcg(A, prec, b, tol, W=None, maxit=80):
    if W is not None:
        AW = A @ W
        Einv = np.linalg.inv(W.conj().T @ AW)
        x = W @ (Einv @ (W.conj().T @ b))
    else:
        x = np.zeros_like(b)
    r = b - A @ x
    bn = np.linalg.norm(b)
    z = prec(r)
    solves = 1
    if W is not None:
        z = z - W @ (Einv @ (AW.conj().T @ z))
    p = z.copy()
    rz = np.vdot(r, z)
    for _ in range(maxit):
        q = A @ p
        a = rz / np.vdot(p, q)
        x = x + a * p
        r = r - a * q
        if np.linalg.norm(r) <= tol * bn:
            return x, solves
        z = prec(r)
        solves += 1
        if W is not None:
            z = z - W @ (Einv @ (AW.conj().T @ z))
        rz2 = np.vdot(r, z)
        p = z + (rz2 / rz) * p
        rz = rz2
    return x, solves


def test_deflated_refinement_matches_and_saves_solves(oracle):
    from turbomodal_gb300.meshgen import TITANIUM, sector_mesh

    mesh = sector_mesh(8, 5, 2, num_sectors=36, jitter=0.02, seed=5,
                       blade=dict(ns=6, nc=3, nb=2, span=0.12, chord=0.05, thick=0.004, twist_deg=30.0))

    def operator(rpm):
        om = oracle.OracleModel(mesh, TITANIUM)
        om.prepare(rpm)
        return om.matrix("Kk", k=1).toarray(), om.matrix("Mk", k=1).toarray()

    K, M = operator(10000.0)
    A = K - M
    s = 1.0 / np.sqrt(np.abs(np.real(np.diag(A))))
    L32 = np.linalg.cholesky(((A * s[:, None]) * s[None, :]).astype(np.complex64))

    def prec(r):                    # F^-1 r with the FP32 factor of S A S: x = S (S A S)^-1 S r
        y = sl.solve_triangular(L32, (s * r).astype(np.complex64), lower=True)
        y = sl.solve_triangular(L32.conj().T, y, lower=False)
        return s * y.astype(np.complex128)

    K2, M2 = operator(6000.0)
    _, V = sl.eigh(K2, M2, subset_by_index=[0, 7])     # lowest eigenvectors at another speed
    rng = np.random.default_rng(3)
    plain, defl = [], []
    for _ in range(4):
        v = rng.standard_normal(len(A)) + 1j * rng.standard_normal(len(A))
        b = M @ v
        x_ref = np.linalg.solve(A, b)
        x0, n0 = pcg(A, prec, b, 1e-10)
        x1, n1 = pcg(A, prec, b, 1e-10, V.astype(complex))
        for x in (x0, x1):   # the recursive residual meets 1e-10; the true one within 10x of it
            assert np.linalg.norm(A @ x - b) <= 1e-9 * np.linalg.norm(b)
            assert np.linalg.norm(x - x_ref) <= 1e-6 * np.linalg.norm(x_ref)
        plain.append(n0)
        defl.append(n1)
    assert np.mean(defl) < np.mean(plain)
