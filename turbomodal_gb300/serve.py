"""Served request stream: concurrent cyclic modal solves on one GPU, admitted by a
device-memory budget, with requests on the same sector batched together.

Every request (sector mesh, material, speed, modes, harmonic subset, precision) runs on a
device context, which owns a non-blocking CUDA stream, its factors and its Lanczos bases.
Worker threads take requests in arrival order.  A worker that takes a request also takes every
queued request on the same sector and precision (continuous batching: requests that arrived
while the GPU was busy join the next batch) and solves them as one batched sweep
(solve_rpm_sweep: the harmonics of all their speeds factorised and iterated together), with the
union of their harmonic subsets and the largest mode count; each request then gets its own
harmonics and its own number of modes from the batch.

Admission by budget covers every device byte a request holds: before its context builds
anything, the request reserves an estimate of the sector set-up (assembly, prestress,
projections, symbolic analyses; bytes per node learnt from earlier contexts), trued up to the
context's own count (tmg_device_bytes) once the set-up is done; then it reserves its
factorisation batch.  Requests wait until that much of the budget is free.

Contexts outlive their requests: an idle context is kept per sector (mesh, boundary data and
material, by content), and a later request on the same sector takes it over with its
assembled sector matrices, structural operator patterns and symbolic analyses.  Idle contexts
stay counted against the budget; when a request cannot be admitted, idle contexts are closed,
least recently used first, before it waits.  The reference solves one request at a time on the
CPU (python/turbomodal/solver.py:237-375); this layer has no counterpart there.
"""

from __future__ import annotations

import copy
import hashlib
import math
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
    batched: int = 1               # requests solved in the same batched sweep

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
    """Concurrent request loop with admission by device-memory budget, batching of queued
    requests on the same sector, and reuse of a sector's context across requests."""

    def __init__(self, device: int = 0, budget_bytes: int = 150 << 30, max_inflight: int = 4,
                 max_cached: int = 8, solver_factory=None, max_batch: int = 8):
        self.device = device
        self.budget = int(budget_bytes)
        self.max_inflight = max_inflight
        self.max_cached = max_cached
        self.max_batch = max_batch
        self._factory = solver_factory or (lambda mesh, material, precision: CyclicSymmetrySolver(
            mesh, material, device=device, precision=precision, mem_budget_bytes=self.budget))
        self._used = 0                      # active grants + bytes of idle contexts
        self._cv = threading.Condition()
        self._idle: OrderedDict = OrderedDict()   # sector key -> [(solver, bytes)], least recently used first
        self.bytes_per_node = 60 << 10      # set-up estimate, raised to what contexts report

    # -- context reuse ------------------------------------------------------------------
    def _checkout(self, key: str):
        """An idle context of this sector and the bytes it holds (still counted), or None."""
        with self._cv:
            lst = self._idle.get(key)
            if lst:
                solver, held = lst.pop()
                if not lst:
                    del self._idle[key]
                return solver, held
        return None, 0

    def _checkin(self, key: str, solver, held: int) -> None:
        """Keep an idle context (its bytes stay counted); beyond max_cached the least recently
        used ones are closed."""
        evicted = []
        with self._cv:
            self._idle.setdefault(key, []).append((solver, held))
            self._idle.move_to_end(key)
            while sum(len(v) for v in self._idle.values()) > self.max_cached:
                evicted.append(self._pop_lru())
        self._close(evicted)

    def _pop_lru(self):
        k0, lst = next(iter(self._idle.items()))
        item = lst.pop(0)
        if not lst:
            del self._idle[k0]
        return item

    def _close(self, items) -> None:
        for solver, held in items:
            solver.close()
            with self._cv:
                self._used -= held
                self._cv.notify_all()

    def cached_contexts(self) -> int:
        with self._cv:
            return sum(len(v) for v in self._idle.values())

    def close(self) -> None:
        """Release every idle context."""
        with self._cv:
            items = [it for lst in self._idle.values() for it in lst]
            self._idle.clear()
        self._close(items)

    # -- memory admission ------------------------------------------------------------
    def _acquire(self, need: int) -> int:
        """Reserve `need` bytes (at most the budget); idle contexts are closed, least recently
        used first, while the reservation does not fit; then wait for active ones."""
        need = max(0, min(int(need), self.budget))
        while True:
            victim = None
            with self._cv:
                if self._used + need <= self.budget:
                    self._used += need
                    return need
                if self._idle:
                    victim = self._pop_lru()
                else:
                    self._cv.wait()
                    continue
            self._close([victim])

    def _acquire_flexible(self, want: int, minimum: int) -> int:
        """Reserve up to `want` bytes, taking what is free once at least `minimum` is (idle contexts
        are closed first, least recently used first).  A batch reservation is flexible because
        the engine sizes its factorisation batches to the grant: two requests that each hold a
        set-up reservation and wait for their batch can therefore never block each other while
        the set-ups and one problem fit the budget."""
        want = max(0, min(int(want), self.budget))
        minimum = max(0, min(int(minimum), want))
        while True:
            victim = None
            with self._cv:
                free = self.budget - self._used
                if free >= want or (free >= minimum and not self._idle):
                    g = max(minimum, min(want, free))
                    self._used += g
                    return g
                if self._idle:
                    victim = self._pop_lru()
                else:
                    self._cv.wait()
                    continue
            self._close([victim])

    def _release(self, grant: int) -> None:
        with self._cv:
            self._used -= grant
            self._cv.notify_all()

    def _resize(self, grant: int, need: int) -> int:
        """Adjust a reservation to `need` bytes (waits if it grows)."""
        if need > grant:
            return grant + self._acquire(need - grant)
        self._release(grant - need)
        return need

    # -- one batch of requests on the same sector ---------------------------------------
    def _run(self, group: list, t0: float) -> list:
        outs = [Completed(r.rid, arrival=r.arrival, start=time.perf_counter() - t0) for r in group]
        req = group[0]
        solver = None
        setup = grant = 0
        key = sector_key(req.mesh, req.material)
        ok = False
        try:
            solver, setup = self._checkout(key)
            reused = solver is not None
            if not reused:   # reserve the set-up before the context allocates anything
                setup = self._acquire(self.bytes_per_node * req.mesh.num_nodes())
                solver = self._factory(req.mesh, req.material, req.precision)
            for o in outs:
                o.reused = reused
            solver.set_memory_budget(self.budget)
            solver.prepare(req.rpm)
            cur, _ = solver.device_bytes()
            self.bytes_per_node = max(self.bytes_per_node, int(1.1 * cur / max(1, req.mesh.num_nodes())))
            setup = self._resize(setup, cur)
            full = list(range(req.mesh.num_sectors // 2 + 1))
            ks = sorted({k for r in group for k in (r.harmonics or full)})
            nm = max(r.num_modes for r in group)
            n_cplx = sum(1 for k in ks if 0 < k and 2 * k != req.mesh.num_sectors)
            stats = solver.symbolic_stats(0)
            need = batch_bytes(stats, nm, max(n_cplx, 2) * len(group), req.precision)
            grant = self._acquire_flexible(min(need, self.budget - setup), batch_bytes(stats, nm, 1, req.precision))
            adm = time.perf_counter() - t0
            for o in outs:
                o.admitted = adm
                o.grant_bytes = grant
            solver.set_memory_budget(grant)
            sweep = solver.solve_rpm_sweep([r.rpm for r in group], nm, ks, precision=req.precision)
            for r, o, res in zip(group, outs, sweep):
                mine = set(r.harmonics or full)
                o.results = [_first_modes(x, r.num_modes) for x in res if x.harmonic_index in mine]
                o.batched = len(group)
            ok = True
        except Exception as e:  # a failed batch is reported, the stream goes on
            for o in outs:
                o.error = f"{type(e).__name__}: {e}"
        finally:
            if grant:
                self._release(grant)
            if solver is not None:
                if ok:
                    cur, _ = solver.device_bytes()
                    setup = self._resize(setup, cur)   # the idle context's bytes stay counted
                    self._checkin(key, solver, setup)
                else:   # a context that failed mid-request is not kept
                    self._close([(solver, setup)])
            elif setup:
                self._release(setup)
            done = time.perf_counter() - t0
            for o in outs:
                o.done = done
        return outs

    # -- the stream -------------------------------------------------------------------
    def serve(self, requests: list, deadline_s: float | None = None) -> list:
        """Replay `requests` at their arrival times; return one Completed per request.  With
        `deadline_s`, no batch starts later than that many seconds after the start: requests
        still queued then are returned with an error ("not started") and count as failed."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        pending: list = []
        cv = threading.Condition()
        finished = [False]
        done: list = []
        t0 = time.perf_counter()

        def take():
            """The oldest queued request and the queued requests on its sector and precision."""
            with cv:
                while not pending and not finished[0]:
                    cv.wait()
                if not pending:
                    return None
                if deadline_s is not None and time.perf_counter() - t0 > deadline_s:
                    late = list(pending)
                    pending.clear()
                    now = time.perf_counter() - t0
                    done.extend(Completed(r.rid, arrival=r.arrival, start=now, done=now,
                                          error="not started: serving deadline passed") for r in late)
                    return None
                first = pending.pop(0)
                key = (sector_key(first.mesh, first.material), first.precision)
                group, rest = [first], []
                for r in pending:
                    if len(group) < self.max_batch and (sector_key(r.mesh, r.material), r.precision) == key:
                        group.append(r)
                    else:
                        rest.append(r)
                pending[:] = rest
                return group

        def worker():
            while True:
                g = take()
                if g is None:
                    return
                outs = self._run(g, t0)
                with cv:
                    done.extend(outs)

        ws = [threading.Thread(target=worker, daemon=True) for _ in range(self.max_inflight)]
        for w in ws:
            w.start()
        for r in reqs:
            dt = r.arrival - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            with cv:
                pending.append(r)
                cv.notify()
        with cv:
            finished[0] = True
            cv.notify_all()
        for w in ws:
            w.join()
        now = time.perf_counter() - t0
        done.extend(Completed(r.rid, arrival=r.arrival, start=now, done=now, error="not started: serving deadline passed")
                    for r in pending)
        return sorted(done, key=lambda c: c.rid)


def _first_modes(r, m: int):
    """The result with its first m modes (a batch ran with the largest mode count of its
    requests; the reference truncates to the requested count the same way,
    src/cyclic_solver.cpp:1058-1211)."""
    if len(r.frequencies) <= m:
        return r
    out = copy.copy(r)
    out.frequencies = r.frequencies[:m]
    out.mode_shapes = r.mode_shapes[:, :m]
    out.whirl_direction = r.whirl_direction[:m]
    out.modal_mass_kg = r.modal_mass_kg[:m]
    return out


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
            "reused_contexts": sum(1 for c in done if c.reused),
            "batched_requests": sum(1 for c in done if c.batched > 1)}
