"""ctypes binding of libtmg.so (the C ABI declared in include/turbomodal_gb300.h).

The shared library is built in-tree by ``turbomodal_gb300.build``.  There is no CPU
fallback: if the library or a CUDA device is missing, calls raise.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtmg.so")

TMG_OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "state error", 4: "numerical error",
          5: "out of device memory budget", 6: "device wait timed out"}

MAT = {"K": 0, "M": 1, "Komega": 2, "G": 3, "Ksigma": 4, "Keff": 5,
       "Kcf": 10, "Kpf": 11, "Mcf": 12, "Mpf": 13, "Gcf": 14, "Gpf": 15,
       "K0r": 20, "M0r": 21, "Khr": 22, "Mhr": 23, "Kk": 30, "Mk": 31, "L1": 32, "L2": 33}
PREC = {"fp64": 0, "mixed": 1}
STATIC_SCRATCH_ENTRIES = 524288   # TMG_STATIC_SCRATCH_ENTRIES

EXPORTED = ["tmg_create", "tmg_destroy", "tmg_last_error", "tmg_upload_sector", "tmg_assemble",
            "tmg_prepare", "tmg_projection", "tmg_symbolic", "tmg_solve_at_rpm", "tmg_result_info",
            "tmg_result_copy", "tmg_last_timing", "tmg_symbolic_stats",
            "tmg_set_profiling", "tmg_profile_solve", "tmg_projection_harmonic_static", "tmg_set_memory_budget",
            "tmg_set_option", "tmg_get_option", "tmg_result_modal_mass", "tmg_solve_sweep", "tmg_tuning_report",
            "tmg_device_bytes", "tmg_reset_peak_bytes"]
OPT = {"shift": 0, "deflate": 1, "tensor_cores": 2, "autotune": 3, "refine_tol": 4}


class SectorDesc(C.Structure):
    _fields_ = [("num_nodes", C.c_int32), ("coords", C.POINTER(C.c_double)),
                ("num_elements", C.c_int32), ("connectivity", C.POINTER(C.c_int32)),
                ("E", C.c_double), ("nu", C.c_double), ("rho", C.c_double),
                ("num_sectors", C.c_int32), ("rotation_axis", C.c_int32),
                ("num_left", C.c_int32), ("left_nodes", C.POINTER(C.c_int32)),
                ("num_right", C.c_int32), ("right_nodes", C.POINTER(C.c_int32)),
                ("num_pairs", C.c_int32), ("pairs", C.POINTER(C.c_int32)),
                ("num_constrained", C.c_int32), ("constrained_nodes", C.POINTER(C.c_int32))]


class ResultMeta(C.Structure):
    _fields_ = [("harmonic_index", C.c_int32), ("num_modes", C.c_int32), ("converged", C.c_int32),
                ("iterations", C.c_int32), ("status", C.c_int32), ("rpm", C.c_double),
                ("max_residual", C.c_double), ("refine_residual", C.c_double)]


_lib = None


def load(build_if_missing: bool = True):
    """Load libtmg.so (building it first when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} is missing; run turbomodal_gb300.build.build()")
        from . import build as _b
        _b.build()
    L = C.CDLL(LIB_PATH)
    P = C.c_void_p
    I64P = C.POINTER(C.c_int64)
    I32P = C.POINTER(C.c_int32)
    DP = C.POINTER(C.c_double)
    L.tmg_create.argtypes = [C.c_int, C.c_size_t, C.POINTER(P)]
    L.tmg_destroy.argtypes = [P]
    L.tmg_last_error.argtypes = [P]
    L.tmg_last_error.restype = C.c_char_p
    L.tmg_upload_sector.argtypes = [P, C.POINTER(SectorDesc)]
    L.tmg_assemble.argtypes = [P, C.c_int, C.c_double, I64P, I32P, I32P, DP]
    L.tmg_prepare.argtypes = [P, C.c_double, C.c_int]
    L.tmg_projection.argtypes = [P, C.c_int, C.c_int, I64P, I32P, I32P, I32P, DP]
    L.tmg_symbolic.argtypes = [P, C.c_int, I32P, I32P, I32P, I32P]
    L.tmg_symbolic_stats.argtypes = [P, C.c_int, DP]
    L.tmg_solve_at_rpm.argtypes = [P, C.c_double, C.c_int, I32P, C.c_int, C.c_int, C.c_double, C.c_int, I32P]
    L.tmg_result_info.argtypes = [P, C.c_int, C.POINTER(ResultMeta)]
    L.tmg_result_copy.argtypes = [P, C.c_int, DP, DP, I32P]
    L.tmg_last_timing.argtypes = [P, DP, C.c_int, I64P]
    L.tmg_set_profiling.argtypes = [P, C.c_int]
    L.tmg_profile_solve.argtypes = [P, DP]
    L.tmg_projection_harmonic_static.argtypes = [P, C.c_int, C.c_int, I64P, I32P, I32P, I32P, DP]
    L.tmg_set_memory_budget.argtypes = [P, C.c_size_t]
    L.tmg_set_option.argtypes = [P, C.c_int, C.c_double]
    L.tmg_result_modal_mass.argtypes = [P, C.c_int, DP]
    L.tmg_tuning_report.argtypes = [P, DP, C.c_int, C.POINTER(C.c_int)]
    L.tmg_device_bytes.argtypes = [P, I64P, I64P]
    L.tmg_reset_peak_bytes.argtypes = [P]
    L.tmg_solve_sweep.argtypes = [P, DP, C.c_int, C.c_int, I32P, C.c_int, C.c_int, C.c_double, C.c_int, I32P]
    L.tmg_get_option.argtypes = [P, C.c_int, DP]
    _lib = L
    return L


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


class Context:
    """One device context (tmg_create / tmg_destroy)."""

    def __init__(self, device: int = 0, mem_budget_bytes: int = 0):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.tmg_create(device, mem_budget_bytes, C.byref(h))
        if rc != TMG_OK:
            raise RuntimeError(f"tmg_create failed ({ERRORS.get(rc, rc)}): no usable CUDA device {device}")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.tmg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def check(self, rc: int, what: str):
        if rc != TMG_OK:
            msg = self.L.tmg_last_error(self.h).decode(errors="replace")
            err = ValueError if rc == 1 else RuntimeError
            raise err(f"{what}: {ERRORS.get(rc, rc)}: {msg}")
