"""Host-side mirror of turbomodal's solver interface over the GB300 C ABI.

``CyclicSymmetrySolver.solve_at_rpm`` keeps the reference signature and result semantics
(src/python_bindings.cpp:321-361, src/cyclic_solver.cpp:725-1357); ``solve`` and
``rpm_sweep`` keep ``tm.solve`` / ``tm.rpm_sweep`` (python/turbomodal/solver.py:237-375,
:499-628), including the enriched ``modal_mass_kg`` field.  All numerical work runs in
libtmg.so on the GPU; failed harmonics are omitted with a warning, as in the reference.
"""

from __future__ import annotations

import ctypes as C
import logging
import sys
import time
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

from . import _lib
from .mesh import Mesh
from .meshgen import Material

logger = logging.getLogger(__name__)


class ModalResult:
    """Result of one harmonic index (include/turbomodal/modal_solver.hpp:8-32)."""

    def __init__(self, harmonic_index=0, rpm=0.0, frequencies=None, mode_shapes=None, whirl_direction=None,
                 converged=True):
        self.harmonic_index = int(harmonic_index)
        self.rpm = float(rpm)
        self.frequencies = np.zeros(0) if frequencies is None else frequencies
        self.mode_shapes = np.zeros((0, 0), np.complex128) if mode_shapes is None else mode_shapes
        self.whirl_direction = np.zeros(0, np.int32) if whirl_direction is None else whirl_direction
        self.converged = bool(converged)
        self.iterations = 0
        self.max_residual = 0.0
        self.refine_residual = 0.0
        # full-annulus modal mass per mode (kg), computed on the device with the result
        self.modal_mass_kg = np.zeros(len(self.frequencies))

    def wave_propagation_velocity(self, radius: float) -> np.ndarray:
        k = self.harmonic_index
        if k <= 0:
            return np.zeros_like(self.frequencies)
        return 2.0 * np.pi * self.frequencies * radius / k

    def __repr__(self):
        return (f"ModalResult(k={self.harmonic_index}, rpm={self.rpm}, "
                f"freqs={np.round(self.frequencies, 3).tolist()}, converged={self.converged})")


@dataclass
class SolverProgress:
    """Callback data of solve_at_rpm's progress_cb (include/turbomodal/cyclic_solver.hpp:16-28,
    python/turbomodal/_core.pyi:150-161)."""

    completed: int = 0
    total: int = 0
    harmonic_k: int = 0
    converged: bool = True
    iterations: int = 0
    num_converged: int = 0
    num_modes: int = 0
    max_residual: float = 0.0
    min_freq_hz: float = 0.0
    max_freq_hz: float = 0.0
    elapsed_s: float = 0.0


@dataclass
class ParametricCondition:
    """Operating condition of solve_parametric (include/turbomodal/cyclic_solver.hpp:58-62,
    src/python_bindings.cpp:300-318)."""

    rpm: float = 0.0
    temperature: float = 293.15
    mistuning: list = field(default_factory=list)

    def __repr__(self):
        return f"<ParametricCondition rpm={self.rpm:f} T={self.temperature:f}K mistuning={len(self.mistuning)} blades>"


class CyclicSymmetrySolver:
    """GPU cyclic-symmetry modal solver for one sector mesh and material."""

    def __init__(self, mesh: Mesh, material: Material, fluid=None, apply_hub_constraint: bool = True,
                 device: int = 0, precision: str = "fp64", mem_budget_bytes: int = 0, deflate: bool = False):
        if fluid is not None and getattr(fluid, "type", None) not in (None, 0, "NONE"):
            raise NotImplementedError("fluid coupling is not part of the GPU path")
        self.mesh = mesh
        self.material = material
        self.apply_hub_constraint = bool(apply_hub_constraint)
        self.precision = precision
        self.ctx = _lib.Context(device, mem_budget_bytes)
        hub = mesh.find_node_set("hub_constraint") if apply_hub_constraint else None
        self._keep = dict(
            X=np.ascontiguousarray(mesh.nodes, dtype=np.float64).reshape(-1),
            conn=np.ascontiguousarray(mesh.elements, dtype=np.int32).reshape(-1),
            left=np.asarray(mesh.left_boundary, dtype=np.int32),
            right=np.asarray(mesh.right_boundary, dtype=np.int32),
            pairs=np.asarray(mesh.matched_pairs, dtype=np.int32).reshape(-1),
            hub=np.asarray(hub.node_ids if hub is not None else [], dtype=np.int32),
        )
        k = self._keep
        d = _lib.SectorDesc(
            mesh.num_nodes(), _lib.ptr(k["X"], C.c_double), mesh.num_elements(), _lib.ptr(k["conn"], C.c_int32),
            material.E, material.nu, material.rho, mesh.num_sectors, mesh.rotation_axis,
            len(k["left"]), _lib.ptr(k["left"], C.c_int32), len(k["right"]), _lib.ptr(k["right"], C.c_int32),
            len(mesh.matched_pairs), _lib.ptr(k["pairs"], C.c_int32), len(k["hub"]), _lib.ptr(k["hub"], C.c_int32))
        self.ctx.check(self.ctx.L.tmg_upload_sector(self.ctx.h, C.byref(d)), "tmg_upload_sector")
        if deflate:
            self.set_option("deflate", 1.0)

    def set_option(self, name: str, value: float) -> None:
        """tmg_set_option: "shift" (sigma of the standard path, default 1.0 as the reference's
        src/cyclic_solver.cpp:1017), "deflate" (1 = deflate the mixed refinement CG with the
        previous speed's eigenvectors) or "tensor_cores" (1 = tcgen05 trailing updates in the
        complex FP32 factorisation; default 0, the SIMT updates)."""
        self.ctx.check(self.ctx.L.tmg_set_option(self.ctx.h, _lib.OPT[name], float(value)), "tmg_set_option")

    def device_bytes(self) -> tuple[int, int]:
        """(current, peak) device bytes of this solver's context (tmg_device_bytes)."""
        cur, peak = C.c_int64(), C.c_int64()
        self.ctx.check(self.ctx.L.tmg_device_bytes(self.ctx.h, C.byref(cur), C.byref(peak)), "tmg_device_bytes")
        return cur.value, peak.value

    def reset_peak_bytes(self) -> None:
        self.ctx.check(self.ctx.L.tmg_reset_peak_bytes(self.ctx.h), "tmg_reset_peak_bytes")

    def tuning_report(self) -> list[dict]:
        """Trials of the last supernode-shape tuning (set_option("autotune", 1))."""
        rows = C.c_int()
        self.ctx.check(self.ctx.L.tmg_tuning_report(self.ctx.h, None, 0, C.byref(rows)), "tmg_tuning_report")
        out = np.zeros(9 * max(rows.value, 1))
        self.ctx.check(self.ctx.L.tmg_tuning_report(self.ctx.h, _lib.ptr(out, C.c_double), rows.value, C.byref(rows)),
                       "tmg_tuning_report")
        keys = ("relax", "max_width", "tc_min_rows", "factor_ms", "solve_ms", "score_ms", "l_entries", "supernodes",
                "chosen")
        return [dict(zip(keys, out[9 * r:9 * r + 9].tolist())) for r in range(rows.value)]

    def get_option(self, name: str) -> float:
        v = C.c_double()
        self.ctx.check(self.ctx.L.tmg_get_option(self.ctx.h, _lib.OPT[name], C.byref(v)), "tmg_get_option")
        return v.value

    # --- modal solve -------------------------------------------------------------------
    def solve_at_rpm(self, rpm: float, num_modes_per_harmonic: int, harmonic_indices=(), max_threads: int = 0,
                     include_coriolis: bool = False, min_frequency: float = 0.0, progress_cb=None,
                     allow_condensation: bool = False, memory_reserve_fraction: float = 0.2,
                     precision: str | None = None, shift: float | None = None) -> list[ModalResult]:
        """Modal solve at one speed (src/python_bindings.cpp:332-361).  With include_coriolis,
        harmonics k > 0 solve the Lancaster QEP and carry whirl directions +1 / -1.  Extensions,
        defaulting to the reference's behaviour: `precision`, and `shift` (sigma of the standard
        path for this call; the reference uses 1.0)."""
        if shift is not None:
            old = self.get_option("shift")
            self.set_option("shift", shift)
            try:
                return self.solve_at_rpm(rpm, num_modes_per_harmonic, harmonic_indices, max_threads, include_coriolis,
                                         min_frequency, progress_cb, allow_condensation, memory_reserve_fraction,
                                         precision)
            finally:
                self.set_option("shift", old)
        prec = _lib.PREC[precision or self.precision]
        t_call = time.perf_counter()
        hi = np.asarray(list(harmonic_indices or []), dtype=np.int32)
        nres = C.c_int32()
        L, h = self.ctx.L, self.ctx.h
        rc = L.tmg_solve_at_rpm(h, float(rpm), int(num_modes_per_harmonic),
                                _lib.ptr(hi, C.c_int32) if hi.size else None, int(hi.size),
                                int(include_coriolis), float(min_frequency), prec, C.byref(nres))
        self.ctx.check(rc, "tmg_solve_at_rpm")
        return self._collect(nres.value, progress_cb, t_call)

    def _collect(self, nres: int, progress_cb=None, t_call: float = 0.0, index: list | None = None) -> list[ModalResult]:
        """Copy the context's results to host ModalResults; failed harmonics are reported on
        stderr and omitted, as the reference does (src/cyclic_solver.cpp:1217-1223).  index, if
        given, receives the context's result index of every returned result."""
        L, h = self.ctx.L, self.ctx.h
        out = []
        ndof = self.mesh.num_dof()
        for idx in range(nres):
            meta = _lib.ResultMeta()
            L.tmg_result_info(h, idx, C.byref(meta))
            if meta.status != _lib.TMG_OK:
                detail = L.tmg_last_error(h).decode(errors="replace")
                sys.stderr.write(f"[CyclicSolver] k={meta.harmonic_index} FAILED: "
                                 f"{_lib.ERRORS.get(meta.status, meta.status)} ({detail})\n")
                continue
            m = meta.num_modes
            f = np.zeros(m)
            w = np.zeros(m, np.int32)
            s = np.zeros(2 * ndof * m)
            L.tmg_result_copy(h, idx, _lib.ptr(f, C.c_double), _lib.ptr(s, C.c_double), _lib.ptr(w, C.c_int32))
            r = ModalResult(meta.harmonic_index, meta.rpm, f, s.view(np.complex128).reshape(m, ndof).T.copy(), w,
                            bool(meta.converged))
            r.iterations = meta.iterations
            r.max_residual = meta.max_residual
            r.refine_residual = meta.refine_residual
            mm = np.zeros(m)
            if m:
                self.ctx.check(L.tmg_result_modal_mass(h, idx, _lib.ptr(mm, C.c_double)), "tmg_result_modal_mass")
            r.modal_mass_kg = mm
            if index is not None:
                index.append(idx)
            if not r.converged:
                sys.stderr.write(f"[CyclicSolver] WARNING: k={r.harmonic_index} eigenvalue solve did not fully converge\n")
            out.append(r)
            if progress_cb is not None:
                progress_cb(SolverProgress(completed=len(out), total=nres, harmonic_k=r.harmonic_index,
                                           converged=r.converged, iterations=r.iterations,
                                           num_converged=m if r.converged else 0, num_modes=m,
                                           max_residual=r.max_residual,
                                           min_freq_hz=float(f.min()) if m else 0.0,
                                           max_freq_hz=float(f.max()) if m else 0.0,
                                           elapsed_s=time.perf_counter() - t_call))
        return out

    def solve_parametric(self, conditions, num_modes_per_harmonic: int, harmonic_indices=(), max_threads: int = 0,
                         include_coriolis: bool = False, min_frequency: float = 0.0, allow_condensation: bool = False,
                         memory_reserve_fraction: float = 0.2, progress_cb=None) -> list[list[ModalResult]]:
        """One result list per condition, in order (src/cyclic_solver.cpp:1375-1485).  The
        reference scales K_base by E(T) / E_ref and projects it, but the solve_at_rpm it then
        calls rebuilds K_eff from the unscaled K_base and projects again (:737-820).  So each
        condition's result is solve_at_rpm(condition.rpm), and temperature and mistuning have no
        effect; this mirror returns the same.  progress_cb gets one call per condition
        (harmonic_k = -1)."""
        out = []
        t0 = time.perf_counter()
        for i, cond in enumerate(conditions):
            out.append(self.solve_at_rpm(float(cond.rpm), num_modes_per_harmonic, harmonic_indices, max_threads,
                                         include_coriolis, min_frequency, None, allow_condensation,
                                         memory_reserve_fraction))
            if progress_cb is not None:
                progress_cb(SolverProgress(completed=i + 1, total=len(conditions), harmonic_k=-1, converged=True,
                                           elapsed_s=time.perf_counter() - t0))
        return out

    def solve_rpm_sweep(self, rpm_values, num_modes_per_harmonic: int, harmonic_indices=(), max_threads: int = 0,
                        include_coriolis: bool = False, min_frequency: float = 0.0,
                        precision: str | None = None) -> list[list[ModalResult]]:
        """One result list per speed, in order (src/cyclic_solver.cpp:1359-1373).  On the standard
        path the harmonics of several speeds are factorised and iterated as one batch
        (tmg_solve_sweep); each speed's results equal solve_at_rpm's at that speed."""
        rpms = np.ascontiguousarray(np.asarray(list(rpm_values), dtype=np.float64))
        prec = _lib.PREC[precision or self.precision]
        hi = np.asarray(list(harmonic_indices or []), dtype=np.int32)
        nres = C.c_int32()
        L, h = self.ctx.L, self.ctx.h
        if rpms.size == 0:
            return []
        rc = L.tmg_solve_sweep(h, _lib.ptr(rpms, C.c_double), int(rpms.size), int(num_modes_per_harmonic),
                               _lib.ptr(hi, C.c_int32) if hi.size else None, int(hi.size), int(include_coriolis),
                               float(min_frequency), prec, C.byref(nres))
        self.ctx.check(rc, "tmg_solve_sweep")
        idx = []
        flat = self._collect(nres.value, index=idx)
        per = nres.value // rpms.size   # the context keeps every speed's harmonics, failed ones included
        out = [[] for _ in range(rpms.size)]
        for i, r in zip(idx, flat):
            out[i // per].append(r)
        return out

    def last_timing(self):
        ph = np.zeros(9)
        nl = C.c_int64()
        self.ctx.L.tmg_last_timing(self.ctx.h, _lib.ptr(ph, C.c_double), 9, C.byref(nl))
        return dict(prepare_ms=float(ph[0]), factor_ms=float(ph[1]), lanczos_ms=float(ph[2]), post_ms=float(ph[3]),
                    device_ms=float(ph[4]), solves=int(ph[5]), applies=int(ph[6]), max_refine_iters=int(ph[7]),
                    retried_fp64=int(ph[8]), kernel_launches=nl.value)

    def set_profiling(self, on: bool) -> None:
        self.ctx.check(self.ctx.L.tmg_set_profiling(self.ctx.h, int(on)), "tmg_set_profiling")

    def profile_solve(self) -> dict:
        out = np.zeros(3)
        self.ctx.check(self.ctx.L.tmg_profile_solve(self.ctx.h, _lib.ptr(out, C.c_double)), "tmg_profile_solve")
        return dict(count=int(out[0]), ms=float(out[1]), bytes=float(out[2]))

    # --- matrices (parity / inspection) --------------------------------------------------
    def assemble(self, which: str, rpm: float = 0.0) -> sp.csc_matrix:
        L, h = self.ctx.L, self.ctx.h
        nnz = C.c_int64()
        self.ctx.check(L.tmg_assemble(h, _lib.MAT[which], float(rpm), C.byref(nnz), None, None, None), "tmg_assemble")
        n = self.mesh.num_dof()
        p = np.zeros(n + 1, np.int32)
        i = np.zeros(max(nnz.value, 1), np.int32)
        x = np.zeros(max(nnz.value, 1))
        self.ctx.check(L.tmg_assemble(h, _lib.MAT[which], float(rpm), C.byref(nnz), _lib.ptr(p, C.c_int32),
                                      _lib.ptr(i, C.c_int32), _lib.ptr(x, C.c_double)), "tmg_assemble")
        A = sp.csc_matrix((x[: nnz.value], i[: nnz.value], p), shape=(n, n))
        A.has_sorted_indices = True
        return A

    def prepare(self, rpm: float, coriolis: bool = False) -> None:
        self.ctx.check(self.ctx.L.tmg_prepare(self.ctx.h, float(rpm), int(coriolis)), "tmg_prepare")

    def projection(self, which: str, k: int = 0) -> sp.csc_matrix:
        L, h = self.ctx.L, self.ctx.h
        nnz, n = C.c_int64(), C.c_int32()
        self.ctx.check(L.tmg_projection(h, _lib.MAT[which], k, C.byref(nnz), C.byref(n), None, None, None),
                       "tmg_projection")
        p = np.zeros(n.value + 1, np.int32)
        i = np.zeros(max(nnz.value, 1), np.int32)
        x = np.zeros(2 * max(nnz.value, 1))
        self.ctx.check(L.tmg_projection(h, _lib.MAT[which], k, C.byref(nnz), C.byref(n), _lib.ptr(p, C.c_int32),
                                        _lib.ptr(i, C.c_int32), _lib.ptr(x, C.c_double)), "tmg_projection")
        vals = x[: 2 * nnz.value].view(np.complex128)
        if which in ("K0r", "M0r", "Khr", "Mhr"):
            vals = x[: nnz.value]
        A = sp.csc_matrix((vals.copy(), i[: nnz.value], p), shape=(n.value, n.value))
        A.has_sorted_indices = True
        return A

    def compute_stationary_frame(self, rotating_result, num_sectors: int | None = None) -> "StationaryFrameResult":
        """Stationary-frame frequencies of one result (python_bindings.cpp:402)."""
        return compute_stationary_frame(rotating_result, num_sectors or self.mesh.num_sectors)

    def export_campbell_csv(self, filename: str, results) -> None:
        export_campbell_csv(filename, results, self.mesh.num_sectors)

    def export_zzenf_csv(self, filename: str, results_at_rpm) -> None:
        export_zzenf_csv(filename, results_at_rpm)

    def set_memory_budget(self, nbytes: int) -> None:
        """Device-memory budget of later solves (tmg_set_memory_budget)."""
        self.ctx.check(self.ctx.L.tmg_set_memory_budget(self.ctx.h, int(nbytes)), "tmg_set_memory_budget")

    def close(self) -> None:
        """Release the device context and its memory now."""
        self.ctx.close()

    def symbolic_stats(self, kind: int = 0) -> dict:
        out = np.zeros(10)
        self.ctx.check(self.ctx.L.tmg_symbolic_stats(self.ctx.h, kind, _lib.ptr(out, C.c_double)),
                       "tmg_symbolic_stats")
        keys = ["n", "nnz_l", "supernodes", "levels", "max_front", "l_entries", "flops", "lower_entries",
                "u_entries", "l_stored"]
        return {k: float(v) for k, v in zip(keys, out)}

    def symbolic(self, kind: int = 0):
        """(AMD order, elimination tree, L column counts) of the shift-invert operator."""
        L, h = self.ctx.L, self.ctx.h
        n = C.c_int32()
        self.ctx.check(L.tmg_symbolic(h, kind, C.byref(n), None, None, None), "tmg_symbolic")
        perm = np.zeros(n.value, np.int32)
        par = np.zeros(n.value, np.int32)
        cc = np.zeros(n.value, np.int32)
        self.ctx.check(L.tmg_symbolic(h, kind, C.byref(n), _lib.ptr(perm, C.c_int32), _lib.ptr(par, C.c_int32),
                                      _lib.ptr(cc, C.c_int32)), "tmg_symbolic")
        return perm, par, cc


@dataclass
class EnrichedModalResult:
    """ModalResult plus full-annulus modal mass (python/turbomodal/solver.py:30-53)."""

    _result: ModalResult = field(repr=False)
    modal_mass_kg: np.ndarray

    def __getattr__(self, name):
        return getattr(self._result, name)


def _modal_mass_from_M(M_sector, results, num_sectors):
    """N * Re(phi^H M phi) per mode (python/turbomodal/solver.py:91-103)."""
    out = []
    for r in results:
        shapes = np.asarray(r.mode_shapes)
        if shapes.size == 0:
            out.append(np.zeros(0))
            continue
        M_phi = M_sector @ shapes
        out.append(np.asarray(num_sectors * np.real(np.sum(shapes.conj() * M_phi, axis=0)), dtype=np.float64))
    return out


def _validate(results):
    for r in results:
        f = np.asarray(r.frequencies)
        if f.size and np.any(np.isnan(f)):
            logger.warning("ND=%d: NaN frequencies detected", r.harmonic_index)
        if f.size and np.any(f < 0):
            logger.warning("ND=%d: negative frequencies detected", r.harmonic_index)
    return results


SILENT = 0
PROGRESS = 1
DETAILED = 2


def _header(mesh, hi, include_coriolis, temperature):
    nd = f"ND {hi}" if hi else f"ND 0..{mesh.num_sectors // 2}"
    cor = " [Coriolis]" if include_coriolis else ""
    tmp = f"  T={temperature:.1f}K" if temperature is not None else ""
    return nd, cor, tmp


def _unsupported(boundary_conditions):
    if boundary_conditions is not None:
        raise NotImplementedError("boundary_conditions (constraint groups) are not on the GPU path")


def solve(mesh: Mesh, material: Material, rpm: float = 0.0, num_modes: int = 20, fluid=None, config=None,
          verbose: int = PROGRESS, harmonic_indices=None, max_threads: int = 0, hub_constraint: str = "fixed",
          include_coriolis: bool = False, min_frequency: float = 0.0, temperature: float | None = None,
          condition=None, boundary_conditions=None, show_convergence: bool = False,
          memory_reserve_fraction: float = 0.2, *, precision: str = "fp64",
          solver: CyclicSymmetrySolver | None = None):
    """tm.solve (python/turbomodal/solver.py:237-375) on the GPU path, with the reference's parameters
    in its order; one EnrichedModalResult per harmonic index.  `condition` supplies rpm and (unless
    given) temperature; `config` is accepted and unused, as in the reference.  Constraint groups
    (`boundary_conditions`) and fluid coupling are not on the GPU path and raise
    NotImplementedError; `show_convergence` (a live plot) is not available and only warns.
    Keyword-only: `precision` ("fp64" or "mixed") and a `solver` to reuse, which must have been
    built for this mesh, material (after `temperature`) and hub constraint (else ValueError)."""
    if condition is not None:
        rpm = condition.rpm
        if temperature is None:
            temperature = condition.temperature
    _unsupported(boundary_conditions)
    if show_convergence:
        logger.warning("show_convergence: no live plot on this path; solving without it")
    if temperature is not None:
        material = material.at_temperature(temperature)
    hi = list(harmonic_indices or [])
    if verbose >= PROGRESS:
        nd, cor, tmp = _header(mesh, hi, include_coriolis, temperature)
        print(f"Solving at {rpm:.0f} RPM{cor}{tmp}  ({mesh.num_nodes()} nodes, {mesh.num_elements()} elements, "
              f"{mesh.num_sectors} sectors, {nd}, {num_modes} modes/ND)")
    t0 = time.perf_counter()
    if solver is not None:
        _check_reused_solver(solver, mesh, material, hub_constraint == "fixed")
    s = solver or CyclicSymmetrySolver(mesh, material, fluid, hub_constraint == "fixed", precision=precision)
    res = s.solve_at_rpm(rpm, num_modes, hi, max_threads, include_coriolis, min_frequency,
                         memory_reserve_fraction=memory_reserve_fraction, precision=precision)
    if verbose >= PROGRESS:
        print(f"  Solved {len(res)} harmonic indices in {time.perf_counter() - t0:.1f}s")
    res = _validate(res)
    out = [EnrichedModalResult(_result=r, modal_mass_kg=r.modal_mass_kg) for r in res]
    if verbose >= DETAILED:
        for r in out:
            freqs = ", ".join(f"{f:.1f}" for f in r.frequencies[:4])
            mm = ", ".join(f"{m:.4e}" for m in r.modal_mass_kg[:4])
            print(f"    ND={r.harmonic_index:2d}: [{freqs}] Hz (rotating frame)")
            print(f"           modal mass [kg]: [{mm}]")
    return out


def _check_reused_solver(solver, mesh, material, apply_hub: bool) -> None:
    """A solver passed to solve() keeps the sector, material and hub constraint it was built
    with; a call asking for different ones (another mesh, a temperature that changes E, another
    hub_constraint) would otherwise be answered for the solver's own, so it is refused."""
    if solver.mesh is not mesh:
        raise ValueError("solve(..., solver=s): s was built for another mesh")
    a, b = solver.material, material
    if not all(np.isclose(getattr(a, f), getattr(b, f), rtol=1e-12, atol=0.0) for f in ("E", "nu", "rho")):
        raise ValueError(f"solve(..., solver=s): s was built for material (E={a.E:g}, nu={a.nu:g}, rho={a.rho:g}); "
                         f"this call asks for (E={b.E:g}, nu={b.nu:g}, rho={b.rho:g}) (temperature or material "
                         "differ); build a new solver")
    if solver.apply_hub_constraint != apply_hub:
        raise ValueError("solve(..., solver=s): s was built with another hub_constraint")


def rpm_sweep(mesh: Mesh, material: Material, rpm_values, num_modes: int = 20, fluid=None, verbose: int = SILENT,
              harmonic_indices=None, max_threads: int = 0, hub_constraint: str = "fixed",
              include_coriolis: bool = False, min_frequency: float = 0.0, temperature: float | None = None,
              boundary_conditions=None, memory_reserve_fraction: float = 0.2, *, precision: str = "fp64"):
    """tm.rpm_sweep (python/turbomodal/solver.py:499-628) on the GPU path, with the reference's
    parameters in its order: one solver (sector assembly and symbolic analysis reused across
    speeds), the speeds solved as batches of several speeds on the device (solve_rpm_sweep), and
    modal masses computed on the device with each result."""
    _unsupported(boundary_conditions)
    if temperature is not None:
        material = material.at_temperature(temperature)
    hi = list(harmonic_indices or [])
    rpms = np.asarray(rpm_values, dtype=np.float64)
    if verbose >= PROGRESS and len(rpms):
        nd, cor, tmp = _header(mesh, hi, include_coriolis, temperature)
        print(f"RPM sweep{cor}{tmp}: {len(rpms)} points [{rpms[0]:.0f} .. {rpms[-1]:.0f}] RPM")
        print(f"  Mesh: {mesh.num_nodes()} nodes, {mesh.num_elements()} elements, {mesh.num_sectors} sectors")
        print(f"  Solving {nd}, {num_modes} modes/ND")
        print()
    s = CyclicSymmetrySolver(mesh, material, fluid, hub_constraint == "fixed", precision=precision)
    out = []
    t_start = time.perf_counter()
    # all speeds in one batched sweep call; the per-speed report follows it
    t0 = time.perf_counter()
    sweep = s.solve_rpm_sweep([float(r) for r in rpms], num_modes, hi, max_threads, include_coriolis, min_frequency,
                              precision=precision)
    for i, rpm in enumerate(rpms):
        res = _validate(sweep[i])
        out.append([EnrichedModalResult(_result=r, modal_mass_kg=r.modal_mass_kg) for r in res])
        if verbose >= DETAILED:
            print(f"  [{i + 1}/{len(rpms)}] {rpm:.0f} RPM  ({len(res)} harmonics, {time.perf_counter() - t0:.1f}s)")
            for r in res:
                freqs = ", ".join(f"{f:.1f}" for f in r.frequencies[:3])
                print(f"      ND={r.harmonic_index:2d}: [{freqs}] Hz")
    if verbose >= PROGRESS and len(rpms):
        total = time.perf_counter() - t_start
        print(f"  Sweep complete in {total:.1f}s ({total / len(rpms):.1f}s/point avg)")
    return out


# --- consumers of a result set (host side) ----------------------------------------------------
@dataclass
class StationaryFrameResult:
    """Stationary-frame frequencies of one rotating-frame result (cyclic_solver.hpp)."""

    frequencies: np.ndarray
    whirl_direction: np.ndarray


def compute_stationary_frame(result, num_sectors: int) -> StationaryFrameResult:
    """Rotating-frame result -> stationary frame (src/cyclic_solver.cpp:374-454): modes that
    carry a whirl direction at speed (k > 0) move by whirl * k * Omega / 2 pi; otherwise, for
    0 < k < N/2 at speed, every mode splits into a forward (f + k Omega / 2 pi) and a backward
    (|f - k Omega / 2 pi|) wave; k = 0, k = N/2 and rest stay standing (whirl 0)."""
    k = int(result.harmonic_index)
    omega = float(result.rpm) * 2.0 * np.pi / 60.0
    f = np.asarray(result.frequencies, dtype=np.float64)
    w = np.asarray(result.whirl_direction, dtype=np.int32)
    kw = k * abs(omega) / (2.0 * np.pi)
    if np.any(w != 0) and abs(omega) > 0.0 and k > 0:
        sf = np.abs(f + w * kw)
        order = np.argsort(sf, kind="stable")
        return StationaryFrameResult(sf[order], w[order])
    if abs(omega) > 0.0 and 0 < k < num_sectors // 2:
        allf = np.empty(2 * len(f))
        allw = np.empty(2 * len(f), dtype=np.int32)
        allf[0::2], allf[1::2] = f + kw, np.abs(f - kw)
        allw[0::2], allw[1::2] = 1, -1
        order = np.argsort(allf, kind="stable")
        return StationaryFrameResult(allf[order], allw[order])
    return StationaryFrameResult(f.copy(), np.zeros(len(f), dtype=np.int32))


def campbell_data(results, num_sectors: int = 0) -> dict:
    """Campbell-diagram arrays from an rpm sweep (python/turbomodal/solver.py:631-744): 'rpm' (N,),
    'frequencies' (N, H, M) stationary-frame Hz (NaN-padded), 'harmonic_index' (H,),
    'whirl_direction' (N, H, M) with +1 forward, -1 backward, 0 standing; M = 2 x the most
    modes of any result.  num_sectors = 0 infers N = 2 x the largest harmonic index."""
    if not results:
        return {"rpm": np.array([]), "frequencies": np.array([]), "harmonic_index": np.array([]),
                "whirl_direction": np.array([])}
    hs = np.array(sorted({r.harmonic_index for row in results for r in row}))
    col = {h: i for i, h in enumerate(hs)}
    if num_sectors <= 0:
        num_sectors = 2 * (int(hs[-1]) if len(hs) else 0)
    max_k = num_sectors // 2
    n_modes = 2 * max((len(r.frequencies) for row in results for r in row), default=0)
    rpm = np.zeros(len(results))
    freqs = np.full((len(results), len(hs), n_modes), np.nan)
    whirl = np.zeros((len(results), len(hs), n_modes), dtype=np.int32)
    for i, row in enumerate(results):
        if row:
            rpm[i] = row[0].rpm
        omega = rpm[i] * 2.0 * np.pi / 60.0
        for r in row:
            j = col.get(r.harmonic_index)
            if j is None:
                continue
            k = r.harmonic_index
            f = np.asarray(r.frequencies, dtype=np.float64)
            w = np.asarray(r.whirl_direction, dtype=np.int32)
            kw = k * abs(omega) / (2.0 * np.pi)
            if np.any(w != 0) and abs(omega) > 0 and k > 0:
                sf = np.abs(f + w * kw)
                order = np.argsort(sf)
                m = min(n_modes, len(f))
                freqs[i, j, :m] = sf[order][:m]
                whirl[i, j, :m] = w[order][:m]
            elif abs(omega) > 0 and 0 < k < max_k:
                allf = np.empty(2 * len(f))
                allw = np.empty(2 * len(f), dtype=np.int32)
                allf[0::2], allf[1::2] = f + kw, np.abs(f - kw)
                allw[0::2], allw[1::2] = 1, -1
                order = np.argsort(allf)
                m = min(n_modes, 2 * len(f))
                freqs[i, j, :m] = allf[order][:m]
                whirl[i, j, :m] = allw[order][:m]
            else:
                m = min(n_modes, len(f))
                freqs[i, j, :m] = f[:m]
    return {"rpm": rpm, "frequencies": freqs, "harmonic_index": hs, "whirl_direction": whirl}


def export_campbell_csv(filename: str, results, num_sectors: int) -> None:
    """rpm,harmonic_index,mode_family,frequency_hz,whirl_direction with stationary-frame
    frequencies, six decimals (src/cyclic_solver.cpp:1487-1506)."""
    with open(filename, "w") as fh:
        fh.write("rpm,harmonic_index,mode_family,frequency_hz,whirl_direction\n")
        for row in results:
            for r in row:
                sf = compute_stationary_frame(r, num_sectors)
                for m, (f, w) in enumerate(zip(sf.frequencies, sf.whirl_direction)):
                    fh.write(f"{r.rpm:.6f},{r.harmonic_index},{m + 1},{f:.6f},{int(w)}\n")


def export_zzenf_csv(filename: str, results_at_rpm) -> None:
    """nodal_diameter,mode_family,frequency_hz,rpm for the results of one speed, six decimals
    (src/cyclic_solver.cpp:1508-1523)."""
    with open(filename, "w") as fh:
        fh.write("nodal_diameter,mode_family,frequency_hz,rpm\n")
        for r in results_at_rpm:
            for m, f in enumerate(r.frequencies):
                fh.write(f"{r.harmonic_index},{m + 1},{f:.6f},{r.rpm:.6f}\n")
