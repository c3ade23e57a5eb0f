"""Served request stream: concurrent cyclic modal solves on one GPU, admitted by a
device-memory budget.

Every request (sector mesh, material, speed, modes, harmonic subset, precision) runs in its
own device context, which owns a non-blocking CUDA stream, its factors and its Lanczos bases
for the life of the request.  Worker threads take requests in arrival order; a request first
builds its operators (assembly, prestress, projections, symbolic analysis), then asks the
server for the device memory its factorisation batch needs and waits until that much of the
budget is free, so requests that arrive while others are on the GPU are admitted as memory
frees up and their kernels overlap on the device.

Contexts outlive their requests: an idle context is kept per sector (mesh, boundary data and
material, by content), and a later request on the same sector takes it over with its
assembled sector matrices, structural operator patterns and symbolic analyses, so only the
speed-dependent work runs again.  At most `max_cached` idle contexts are kept (least recently
used evicted).  The reference solves one request at a time on the CPU
(python/turbomodal/solver.py:237-375); this layer has no counterpart there.
"""

from __future__ import annotations

import hashlib
import math
import queue
import threading
import time
from collections import OrderedDict
from dataclasses import dataclass, field

import numpy as np

from .meshgen import Material
from .solver import CyclicSymmetrySolver


@dataclass
class Request:
    rid: int
    mesh: object
    material: Material
    rpm: float
    num_modes: int
    harmonics: list
    precision: str = "mixed"
    arrival: float = 0.0           # seconds after the start of the stream


@dataclass
class Completed:
    rid: int
    results: list = field(default_factory=list)
    arrival: float = 0.0
    start: float = 0.0
    admitted: float = 0.0
    done: float = 0.0
    grant_bytes: int = 0
    error: str = ""
    reused: bool = False           # ran on a context kept from an earlier request

    @property
    def latency(self) -> float:
        return self.done - self.arrival

    @property
    def eigenpairs(self) -> int:
        return sum(len(r.frequencies) for r in self.results)


def batch_bytes(stats: dict, num_modes: int, nproblems: int, precision: str) -> int:
    """Device memory of one factorisation batch of `nproblems` complex harmonics (the
    estimate the engine uses to size its batches): factor panels and update workspace in the
    factor precision, FP64 operator values and Lanczos bases."""
    n = stats["n"]
    fb = 8.0 if precision == "mixed" else 16.0
    nev = max(1, (num_modes + 1) // 2)
    ncv = min(max(4 * nev + 1, 40), int(n))
    per = (fb * (stats["l_entries"] + stats["u_entries"] + 2.0 * n) + 16.0 * (6.0 * stats["lower_entries"])
           + 16.0 * n * (2.0 * (ncv + 1) + 12.0))
    return int(per * max(1, nproblems) * 1.15 + (256 << 20))


def sector_key(mesh, material, apply_hub_constraint: bool = True) -> str:
    """Content fingerprint of everything a context's sector state depends on: geometry,
    connectivity, cyclic boundary data, hub nodes and material."""
    h = hashlib.sha1()
    hub = mesh.find_node_set("hub_constraint") if apply_hub_constraint else None
    for a in (mesh.nodes, mesh.elements, mesh.left_boundary, mesh.right_boundary, mesh.matched_pairs,
              hub.node_ids if hub is not None else []):
        arr = np.ascontiguousarray(np.asarray(a))
        h.update(str(arr.dtype).encode() + str(arr.shape).encode())
        h.update(arr.tobytes())
    h.update(repr((int(mesh.num_sectors), int(mesh.rotation_axis), float(material.E), float(material.nu),
                   float(material.rho))).encode())
    return h.hexdigest()


class ModalServer:
    """Concurrent request loop with admission by device-memory budget and reuse of a sector's
    context across requests."""

    def __init__(self, device: int = 0, budget_bytes: int = 150 << 30, max_inflight: int = 4,
                 max_cached: int = 8, solver_factory=None):
        self.device = device
        self.budget = int(budget_bytes)
        self.max_inflight = max_inflight
        self.max_cached = max_cached
        self._factory = solver_factory or (lambda mesh, material, precision: CyclicSymmetrySolver(
            mesh, material, device=device, precision=precision, mem_budget_bytes=self.budget))
        self._used = 0
        self._cv = threading.Condition()
        self._idle: OrderedDict = OrderedDict()   # sector key -> idle contexts, least recently used first
        self._pool_lock = threading.Lock()

    # -- context reuse ------------------------------------------------------------------
    def _checkout(self, key: str, mesh, material, precision: str):
        """An idle context of this sector (reused = True) or a new one."""
        with self._pool_lock:
            lst = self._idle.get(key)
            if lst:
                solver = lst.pop()
                if not lst:
                    del self._idle[key]
                return solver, True
        return self._factory(mesh, material, precision), False

    def _checkin(self, key: str, solver) -> None:
        """Keep an idle context; the least recently used ones beyond max_cached are closed."""
        evicted = []
        with self._pool_lock:
            self._idle.setdefault(key, []).append(solver)
            self._idle.move_to_end(key)
            while sum(len(v) for v in self._idle.values()) > self.max_cached:
                k0, lst = next(iter(self._idle.items()))
                evicted.append(lst.pop(0))
                if not lst:
                    del self._idle[k0]
        for s in evicted:
            s.close()

    def cached_contexts(self) -> int:
        with self._pool_lock:
            return sum(len(v) for v in self._idle.values())

    def close(self) -> None:
        """Release every idle context."""
        with self._pool_lock:
            items = [s for lst in self._idle.values() for s in lst]
            self._idle.clear()
        for s in items:
            s.close()

    # -- memory admission ------------------------------------------------------------
    def _acquire(self, need: int) -> int:
        need = min(need, self.budget)
        with self._cv:
            while self._used + need > self.budget:
                self._cv.wait()
            self._used += need
        return need

    def _release(self, grant: int) -> None:
        with self._cv:
            self._used -= grant
            self._cv.notify_all()

    # -- one request ------------------------------------------------------------------
    def _run(self, req: Request, t0: float) -> Completed:
        out = Completed(req.rid, arrival=req.arrival, start=time.perf_counter() - t0)
        solver = None
        grant = 0
        key = sector_key(req.mesh, req.material)
        ok = False
        try:
            solver, out.reused = self._checkout(key, req.mesh, req.material, req.precision)
            solver.set_memory_budget(self.budget)
            solver.prepare(req.rpm)
            ks = list(req.harmonics) or list(range(req.mesh.num_sectors // 2 + 1))
            n_cplx = sum(1 for k in ks if 0 < k and 2 * k != req.mesh.num_sectors)
            need = batch_bytes(solver.symbolic_stats(0), req.num_modes, max(n_cplx, 2), req.precision)
            grant = self._acquire(need)
            out.admitted = time.perf_counter() - t0
            out.grant_bytes = grant
            solver.set_memory_budget(grant)
            out.results = solver.solve_at_rpm(req.rpm, req.num_modes, ks, precision=req.precision)
            ok = True
        except Exception as e:  # a failed request is reported, the stream goes on
            out.error = f"{type(e).__name__}: {e}"
        finally:
            if grant:
                self._release(grant)
            if solver is not None:
                if ok:
                    self._checkin(key, solver)
                else:   # a context that failed mid-request is not kept
                    solver.close()
            out.done = time.perf_counter() - t0
        return out

    # -- the stream -------------------------------------------------------------------
    def serve(self, requests: list) -> list:
        """Replay `requests` at their arrival times; return one Completed per request."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        q: queue.Queue = queue.Queue()
        done: list = []
        lock = threading.Lock()
        t0 = time.perf_counter()

        def worker():
            while True:
                r = q.get()
                if r is None:
                    return
                c = self._run(r, t0)
                with lock:
                    done.append(c)

        ws = [threading.Thread(target=worker, daemon=True) for _ in range(self.max_inflight)]
        for w in ws:
            w.start()
        for r in reqs:
            dt = r.arrival - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            q.put(r)
        for _ in ws:
            q.put(None)
        for w in ws:
            w.join()
        return sorted(done, key=lambda c: c.rid)


def request_stream(n: int, seed: int, rate_hz: float = 20.0, min_nodes: int = 2000, max_nodes: int = 200000,
                   precision: str = "mixed", distinct_sectors: int | None = None) -> list:
    """Seeded request stream: Poisson arrivals at `rate_hz`, config-0/1-style sectors of
    log-uniform size in [min_nodes, max_nodes], 24/36/48 sectors, rpm U(0, 15000), 5..20
    modes, a random subset of 1..19 harmonic indices, titanium.  With `distinct_sectors`,
    every request draws its sector from that many seeded designs (a fleet of repeated
    designs) instead of a new sector per request."""
    from .meshgen import TITANIUM, scaled_mesh

    rng = np.random.default_rng(seed)
    designs = []
    if distinct_sectors:
        for _ in range(distinct_sectors):
            nodes = int(math.exp(rng.uniform(math.log(min_nodes), math.log(max_nodes))))
            ns = int(rng.choice([24, 36, 48]))
            designs.append(scaled_mesh(nodes, ns, seed=int(rng.integers(1 << 30)), with_blade=nodes > 6000))
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate_hz)
        if designs:
            mesh = designs[int(rng.integers(len(designs)))]
            ns = mesh.num_sectors
        else:
            nodes = int(math.exp(rng.uniform(math.log(min_nodes), math.log(max_nodes))))
            ns = int(rng.choice([24, 36, 48]))
            mesh = scaled_mesh(nodes, ns, seed=int(rng.integers(1 << 30)), with_blade=nodes > 6000)
        kmax = ns // 2
        nk = int(rng.integers(1, min(19, kmax + 1) + 1))
        ks = sorted(int(k) for k in rng.choice(kmax + 1, size=nk, replace=False))
        out.append(Request(i, mesh, TITANIUM, float(rng.uniform(0.0, 15000.0)), int(rng.integers(5, 21)), ks,
                           precision, t))
    return out


def latency_summary(done: list) -> dict:
    ok = [c for c in done if not c.error]
    lat = np.array([c.latency for c in ok]) if ok else np.zeros(1)
    span = max((c.done for c in done), default=0.0) - min((c.arrival for c in done), default=0.0)
    pairs = sum(c.eigenpairs for c in ok)
    return {"requests": len(done), "failed": len(done) - len(ok), "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "eigenpairs": pairs,
            "eigenpairs_per_s": pairs / span if span > 0 else 0.0, "makespan_s": span,
            "reused_contexts": sum(1 for c in done if c.reused)}
