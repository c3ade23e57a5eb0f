"""tmg_projection_harmonic_static (per-harmonic K_k / M_k formed in a static device array, no
device allocation) against tmg_projection, through the C ABI.

Collected last (file name) so that it also runs after every other GPU test in one process;
it builds its own context, so it passes alone in a fresh process too.
Tolerance: the two entry points run the same arithmetic, so the values must agree to
1e-15 relative to the matrix's largest entry, and the patterns exactly.  Against the oracle's
K_k / M_k (the reference's per-harmonic sum, src/cyclic_solver.cpp:942-947) the static entry
point's matrix must agree within 1e-12 of the largest entry at 10000 rpm (the prestress solve
differs in its last bits), with the reference's pruned entries present as exact zeros.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-15


@pytest.fixture(scope="module")
def solver():
    from turbomodal_gb300.meshgen import TITANIUM, config_mesh
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    s = CyclicSymmetrySolver(config_mesh(0), TITANIUM)
    s.prepare(10000.0)
    return s


def call(s, fn, which, k):
    from turbomodal_gb300 import _lib

    ctx = s.ctx
    nnz, n = C.c_int64(), C.c_int32()
    ctx.check(fn(ctx.h, which, k, C.byref(nnz), C.byref(n), None, None, None), fn.__name__)
    colptr = np.zeros(n.value + 1, np.int32)
    rowidx = np.zeros(nnz.value, np.int32)
    vals = np.zeros(2 * nnz.value)
    ctx.check(fn(ctx.h, which, k, C.byref(nnz), C.byref(n), _lib.ptr(colptr, C.c_int32), _lib.ptr(rowidx, C.c_int32),
                 _lib.ptr(vals, C.c_double)), fn.__name__)
    return colptr, rowidx, vals


@pytest.mark.parametrize("name,k", [("Kk", 1), ("Mk", 1), ("Kk", 7), ("Mk", 18)])
def test_static_scratch_matches_allocating_entry_point(solver, name, k):
    from turbomodal_gb300 import _lib

    L = solver.ctx.L
    which = _lib.MAT[name]
    ref = call(solver, L.tmg_projection, which, k)
    assert ref[2].size // 2 <= _lib.STATIC_SCRATCH_ENTRIES
    for _ in range(2):   # two calls in a row reuse the same scratch
        got = call(solver, L.tmg_projection_harmonic_static, which, k)
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
        scale = np.abs(ref[2]).max()
        assert np.abs(got[2] - ref[2]).max() <= TOL * scale


def test_static_scratch_rejects_oversize_matrix():
    from turbomodal_gb300 import _lib
    from turbomodal_gb300.meshgen import STEEL, sector_mesh
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    s = CyclicSymmetrySolver(sector_mesh(16, 10, 3, seed=2), STEEL)
    s.prepare(0.0)
    nnz, n = C.c_int64(), C.c_int32()
    rc = s.ctx.L.tmg_projection_harmonic_static(s.ctx.h, _lib.MAT["Kk"], 1, C.byref(nnz), C.byref(n), None, None, None)
    assert rc == 1
    assert nnz.value > _lib.STATIC_SCRATCH_ENTRIES
    assert "static scratch" in s.ctx.L.tmg_last_error(s.ctx.h).decode()
    with pytest.raises(ValueError):
        s.ctx.check(s.ctx.L.tmg_projection_harmonic_static(s.ctx.h, _lib.MAT["Kk"], 2, C.byref(nnz), C.byref(n),
                                                           None, None, None), "tmg_projection_harmonic_static")


@pytest.mark.parametrize("name,k", [("Kk", 1), ("Mk", 5), ("Kk", 18)])
def test_static_scratch_matches_oracle(solver, oracle, name, k):
    import scipy.sparse as sp

    from turbomodal_gb300 import _lib
    from turbomodal_gb300.meshgen import TITANIUM, config_mesh

    colptr, rowidx, vals = call(solver, solver.ctx.L.tmg_projection_harmonic_static, _lib.MAT[name], k)
    n = colptr.size - 1
    got = sp.csc_matrix((vals.view(np.complex128), rowidx, colptr), shape=(n, n))
    om = oracle.OracleModel(config_mesh(0), TITANIUM)
    om.prepare(10000.0)
    ref = om.matrix(name, k=k)
    assert ref.shape == got.shape
    scale = abs(ref).max()
    assert abs(got - ref).max() <= 1e-12 * scale
    # every entry of the reference's pattern is in the static entry point's pattern
    onlyref = abs(ref).multiply(abs(got) == 0)
    assert onlyref.nnz == 0 or onlyref.max() <= 1e-12 * scale
