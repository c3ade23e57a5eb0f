"""Oracle (test infrastructure only): ctypes wrapper over the CPU restatement (liborc.so).

Imported by tests/, by the smoke check and by the bench's CPU-baseline leg.  The product
package never imports it.  Build with ``make -C oracle`` (``build()`` in
``__graft_entry__`` does this).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np
import scipy.sparse as sp

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_I = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_D = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(quiet: bool = True) -> str:
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(_HERE, "liborc.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liborc.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.orc_model_create.restype = C.c_void_p
        L.orc_model_create.argtypes = [C.c_int, _D, C.c_int, _I, C.c_double, C.c_double, C.c_double,
                                       C.c_int, C.c_int, C.c_int, _I, C.c_int, _I, C.c_int, _I, C.c_int, _I]
        L.orc_model_free.argtypes = [C.c_void_p]
        L.orc_element.argtypes = [_D, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_int, _D, _D]
        L.orc_prepare.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.orc_prepare.restype = C.c_int
        L.orc_matrix.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int]
        L.orc_matrix.restype = C.c_longlong
        L.orc_matrix_shape.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.orc_matrix_copy.argtypes = [C.c_void_p, _I, _I, _D]
        L.orc_centrifugal.argtypes = [C.c_void_p, C.c_double, _D]
        L.orc_static_u.argtypes = [C.c_void_p, _D]
        L.orc_static_u.restype = C.c_int
        L.orc_free_map.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_free_map.restype = C.c_int
        L.orc_ldl_symbolic.argtypes = [C.c_int, _I, _I, _I, _I, _I]
        L.orc_lanczos_z.argtypes = [C.c_int, _I, _I, _D, _I, _I, _D, C.c_int, C.c_int, C.c_double,
                                    C.c_double, C.c_int, _D, _D, _I]
        L.orc_lanczos_z.restype = C.c_int
        L.orc_solve.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, _I, C.c_int, C.c_int, C.c_double]
        L.orc_solve.restype = C.c_int
        L.orc_result_info.argtypes = [C.c_void_p, C.c_int, _I, C.POINTER(C.c_double)]
        L.orc_result_copy.argtypes = [C.c_void_p, C.c_int, _D, C.c_void_p, _I]
        L.orc_lw_create.restype = C.c_void_p
        L.orc_lw_create.argtypes = [C.c_int, _I, _I, _D]
        L.orc_lw_add_slot.restype = C.c_int
        L.orc_lw_add_slot.argtypes = [C.c_void_p]
        L.orc_lw_free.argtypes = [C.c_void_p]
        L.orc_lw_info.argtypes = [C.c_void_p, _D]
        L.orc_lw_cumwork.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")]
        L.orc_lw_run.argtypes = [C.c_void_p, C.c_int, _I, _I, _I, _D, C.c_void_p]
        _LIB = L
    return _LIB


MATRIX_CODES = {"K": 0, "M": 1, "Komega": 2, "G": 3, "Ksigma": 4, "Keff": 5, "T": 6,
                "Kcf": 10, "Kpf": 11, "Mcf": 12, "Mpf": 13, "Gcf": 14, "Gpf": 15,
                "K0r": 20, "M0r": 21, "Khr": 22, "Mhr": 23, "Kk": 30, "Mk": 31, "Gk": 32}


def element(X10x3, mat, kind: int, omega: float = 0.0, axis: int = 2, ue=None):
    X = np.ascontiguousarray(X10x3, dtype=np.float64).reshape(30)
    out = np.zeros(30 if kind == 5 else 900, dtype=np.float64)
    u = np.zeros(30) if ue is None else np.ascontiguousarray(ue, dtype=np.float64)
    lib().orc_element(X, mat.E, mat.nu, mat.rho, kind, omega, axis, u, out)
    return out if kind == 5 else out.reshape(30, 30)


class OracleModel:
    """CPU restatement of CyclicSymmetrySolver on one mesh + material."""

    def __init__(self, mesh, mat, apply_hub: bool = True):
        L = lib()
        hub = mesh.find_node_set("hub_constraint")
        hub_ids = np.asarray(hub.node_ids if (apply_hub and hub is not None) else [], dtype=np.int32)
        pairs = np.asarray(mesh.matched_pairs, dtype=np.int32).reshape(-1)
        self.mesh = mesh
        self._h = L.orc_model_create(
            mesh.num_nodes(), np.ascontiguousarray(mesh.nodes, dtype=np.float64).reshape(-1),
            mesh.num_elements(), np.ascontiguousarray(mesh.elements, dtype=np.int32).reshape(-1),
            mat.E, mat.nu, mat.rho, mesh.num_sectors, mesh.rotation_axis,
            len(mesh.left_boundary), np.asarray(mesh.left_boundary, dtype=np.int32),
            len(mesh.right_boundary), np.asarray(mesh.right_boundary, dtype=np.int32),
            len(mesh.matched_pairs), pairs if pairs.size else np.zeros(1, np.int32),
            len(hub_ids), hub_ids if hub_ids.size else np.zeros(1, np.int32))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_model_free(self._h)
            self._h = None

    def prepare(self, rpm: float, coriolis: bool = False) -> None:
        if lib().orc_prepare(self._h, rpm, int(coriolis)) != 0:
            raise RuntimeError("oracle prepare failed")

    def matrix(self, name: str, param: float = 0.0, k: int = 0) -> sp.csc_matrix:
        L = lib()
        nnz = L.orc_matrix(self._h, MATRIX_CODES[name], param, k)
        if nnz < 0:
            raise RuntimeError(f"oracle matrix {name} failed")
        r, c, z = C.c_int(), C.c_int(), C.c_int()
        L.orc_matrix_shape(self._h, C.byref(r), C.byref(c), C.byref(z))
        p = np.zeros(c.value + 1, np.int32)
        i = np.zeros(max(nnz, 1), np.int32)
        x = np.zeros(max(nnz, 1) * (2 if z.value else 1), np.float64)
        L.orc_matrix_copy(self._h, p, i, x)
        vals = x[: 2 * nnz].view(np.complex128) if z.value else x[:nnz]
        A = sp.csc_matrix((vals.copy(), i[:nnz].copy(), p), shape=(r.value, c.value))
        A.has_sorted_indices = True
        return A

    def centrifugal(self, omega: float) -> np.ndarray:
        F = np.zeros(self.mesh.num_dof())
        lib().orc_centrifugal(self._h, omega, F)
        return F

    def static_u(self) -> np.ndarray:
        u = np.zeros(self.mesh.num_dof())
        if lib().orc_static_u(self._h, u) != 0:
            raise RuntimeError("no static solution (rpm == 0 or free hub)")
        return u

    def free_map(self) -> np.ndarray:
        n = lib().orc_free_map(self._h, None)
        out = np.zeros(max(n, 1), np.int32)
        lib().orc_free_map(self._h, out.ctypes.data)
        return out[:n]

    def solve(self, rpm: float, num_modes: int, harmonic_indices=(), max_threads: int = 0,
              include_coriolis: bool = False, min_frequency: float = 0.0, with_shapes: bool = True):
        L = lib()
        hi = np.asarray(list(harmonic_indices), dtype=np.int32)
        n = L.orc_solve(self._h, rpm, num_modes, len(hi), hi if hi.size else np.zeros(1, np.int32),
                        max_threads, int(include_coriolis), min_frequency)
        if n < 0:
            raise RuntimeError("oracle solve failed")
        out = []
        ndof = self.mesh.num_dof()
        for idx in range(n):
            info = np.zeros(4, np.int32)
            rpm_c = C.c_double()
            L.orc_result_info(self._h, idx, info, C.byref(rpm_c))
            m = int(info[1])
            f = np.zeros(max(m, 1))
            w = np.zeros(max(m, 1), np.int32)
            shp = np.zeros(2 * ndof * max(m, 1)) if with_shapes else None
            L.orc_result_copy(self._h, idx, f, shp.ctypes.data if with_shapes else None, w)
            res = dict(harmonic_index=int(info[0]), rpm=rpm_c.value, frequencies=f[:m].copy(),
                       whirl_direction=w[:m].copy(), converged=bool(info[2]), iterations=int(info[3]))
            if with_shapes:
                res["mode_shapes"] = shp[: 2 * ndof * m].view(np.complex128).reshape(m, ndof).T.copy()
            out.append(res)
        return out


def ldl_symbolic(A_lower: sp.csc_matrix):
    """AMD order, elimination tree and L column counts of a Hermitian pattern (lower triangle)."""
    A = sp.csc_matrix(A_lower)
    A.sort_indices()
    n = A.shape[0]
    perm = np.zeros(n, np.int32)
    parent = np.zeros(n, np.int32)
    cc = np.zeros(n, np.int32)
    lib().orc_ldl_symbolic(n, A.indptr.astype(np.int32), A.indices.astype(np.int32), perm, parent, cc)
    return perm, parent, cc


def lanczos(K: sp.csc_matrix, M: sp.csc_matrix, nev: int, ncv: int = 0, shift: float = 0.0,
            tol: float = 1e-8, maxit: int = 10):
    """Reference Hermitian Lanczos on caller matrices; returns (eigenvalues, vectors, info)."""
    K = sp.csc_matrix(K, dtype=np.complex128)
    M = sp.csc_matrix(M, dtype=np.complex128)
    K.sort_indices(); M.sort_indices()
    n = K.shape[0]
    ev = np.zeros(max(nev, 1))
    vec = np.zeros(2 * n * max(nev, 1))
    info = np.zeros(4, np.int32)
    kx = np.ascontiguousarray(K.data).view(np.float64)
    mx = np.ascontiguousarray(M.data).view(np.float64)
    lib().orc_lanczos_z(n, K.indptr.astype(np.int32), K.indices.astype(np.int32), kx,
                        M.indptr.astype(np.int32), M.indices.astype(np.int32), mx, nev, ncv, shift, tol,
                        maxit, ev, vec, info)
    m = int(info[0])
    return ev[:m], vec[: 2 * n * m].view(np.complex128).reshape(m, n).T, info


def _lower_z(A):
    A = sp.csc_matrix(sp.tril(sp.csc_matrix(A, dtype=np.complex128)))
    A.sort_indices()
    return (A.shape[0], A.indptr.astype(np.int32), A.indices.astype(np.int32),
            np.ascontiguousarray(A.data).view(np.float64))


class LdlWindows:
    """Timing samples of the reference's up-looking LDL^H (Eigen SimplicialLDLT, restated in
    orc_amd.hpp) on one operator: the complete structure of L from the symbolic analysis, one
    slot of L values per thread, row windows of the numeric loop and whole solves timed on
    concurrent threads (orc_window.hpp)."""

    def __init__(self, A):
        n, p, i, x = _lower_z(A)
        self._h = lib().orc_lw_create(n, p, i, x)
        if not self._h:
            raise RuntimeError("orc_lw_create failed")
        info = self.info()
        self.n = int(info[0])
        self.nnz_l = int(info[1])
        self.total_work = int(info[2])

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_lw_free(self._h)
            self._h = None

    def add_slot(self) -> int:
        """One more slot (own L values, shared operator); returns the number of slots."""
        r = lib().orc_lw_add_slot(self._h)
        if r < 0:
            raise MemoryError("orc_lw_add_slot failed")
        return r

    def info(self) -> np.ndarray:
        out = np.zeros(4)
        lib().orc_lw_info(self._h, out)
        return out

    def cumwork(self) -> np.ndarray:
        cum = np.zeros(self.n + 1, np.int64)
        lib().orc_lw_cumwork(self._h, cum)
        return cum

    def run(self, slots, a, b, solve: bool = True):
        """Concurrent samples: thread t times rows [a[t], b[t]) of the numeric loop on slot
        slots[t], then (solve=True) one solve; returns (factor seconds, solve seconds)."""
        slots = np.ascontiguousarray(slots, dtype=np.int32)
        a = np.ascontiguousarray(a, dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=np.int32)
        tf = np.zeros(len(slots))
        ts = np.zeros(len(slots))
        lib().orc_lw_run(self._h, len(slots), slots, a, b, tf, ts.ctypes.data if solve else None)
        return tf, ts
