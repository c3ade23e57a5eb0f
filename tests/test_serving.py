"""Served request stream: admission by device-memory budget, idle-context accounting and
batching of same-sector requests (host logic, CPU) and, on the GPU, concurrent requests whose
results equal the same requests solved alone.

Tolerance: frequencies of a request in the mix within 1e-8 relative of the request alone.  A
request batched with others on its sector is solved with the union of their harmonics and the
largest mode count (a larger Lanczos subspace), so its eigenvalues agree to the Lanczos
convergence tolerance rather than to the last bit; 1e-6 is the parity bar."""

import threading
import time

import numpy as np
import pytest


def test_admission_respects_budget():
    from turbomodal_gb300.serve import ModalServer

    srv = ModalServer(budget_bytes=100, max_inflight=4)
    live, peak = [0], [0]
    lock = threading.Lock()

    def job(need):
        g = srv._acquire(need)
        with lock:
            live[0] += g
            peak[0] = max(peak[0], live[0])
        time.sleep(0.02)
        with lock:
            live[0] -= g
        srv._release(g)

    ts = [threading.Thread(target=job, args=(n,)) for n in (60, 30, 50, 40, 250, 10)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert peak[0] <= 100 and srv._used == 0


def test_request_stream_is_seeded():
    from turbomodal_gb300.serve import request_stream

    a = request_stream(4, seed=5, max_nodes=8000)
    b = request_stream(4, seed=5, max_nodes=8000)
    assert [(r.rpm, r.harmonics, r.num_modes, r.arrival) for r in a] == [(r.rpm, r.harmonics, r.num_modes, r.arrival)
                                                                           for r in b]
    assert all(np.array_equal(x.mesh.nodes, y.mesh.nodes) for x, y in zip(a, b))
    assert all(a[i].arrival < a[i + 1].arrival for i in range(3))


@pytest.mark.gpu
def test_each_result_same_alone_and_in_the_mix():
    from turbomodal_gb300.serve import ModalServer, request_stream
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    reqs = request_stream(6, seed=3, rate_hz=50.0, min_nodes=2000, max_nodes=12000)
    done = ModalServer(budget_bytes=24 << 30, max_inflight=3).serve(reqs)
    assert all(not c.error for c in done), [c.error for c in done]
    spans = sorted((c.admitted, c.done) for c in done)
    assert any(spans[i + 1][0] < spans[i][1] for i in range(len(spans) - 1)), "no two requests overlapped"
    for r, c in zip(sorted(reqs, key=lambda r: r.rid), done):
        s = CyclicSymmetrySolver(r.mesh, r.material, precision=r.precision)
        alone = {x.harmonic_index: x for x in s.solve_at_rpm(r.rpm, r.num_modes, r.harmonics, precision=r.precision)}
        s.close()
        mixed = {x.harmonic_index: x for x in c.results}
        assert sorted(alone) == sorted(mixed)
        for k, a in alone.items():
            assert len(mixed[k].frequencies) == len(a.frequencies)
            np.testing.assert_allclose(mixed[k].frequencies, a.frequencies, rtol=1e-8)


def test_sector_key_tracks_sector_content():
    import copy
    import dataclasses

    from turbomodal_gb300.meshgen import TITANIUM, sector_mesh
    from turbomodal_gb300.serve import sector_key

    a = sector_mesh(4, 3, 1, num_sectors=24, seed=1)
    b = copy.deepcopy(a)
    assert sector_key(a, TITANIUM) == sector_key(b, TITANIUM)
    assert sector_key(a, TITANIUM) != sector_key(a, dataclasses.replace(TITANIUM, E=TITANIUM.E * 1.01))
    b.nodes = b.nodes.copy()
    b.nodes[5, 0] += 1e-9
    assert sector_key(a, TITANIUM) != sector_key(b, TITANIUM)
    c = sector_mesh(4, 3, 1, num_sectors=36, seed=1)
    assert sector_key(a, TITANIUM) != sector_key(c, TITANIUM)


def test_context_pool_reuse_and_eviction():
    """Idle contexts are handed to later requests on the same sector with the bytes they hold
    (still counted against the budget); beyond max_cached the least recently used are closed and
    their bytes returned; an admission that does not fit closes idle contexts first."""
    from turbomodal_gb300.serve import ModalServer

    closed = []

    class Fake:
        def __init__(self, tag):
            self.tag = tag

        def close(self):
            closed.append(self.tag)

    srv = ModalServer(budget_bytes=100, max_cached=2)
    assert srv._checkout("A") == (None, 0)
    a1, a2, b1 = Fake("a1"), Fake("a2"), Fake("b1")
    for s, key in ((a1, "A"), (a2, "A"), (b1, "B")):
        srv._acquire(20)
        srv._checkin(key, s, 20)
    assert closed == ["a1"] and srv.cached_contexts() == 2 and srv._used == 40
    s, held = srv._checkout("A")
    assert s is a2 and held == 20 and srv.cached_contexts() == 1
    srv._checkin("A", s, held)
    g = srv._acquire(90)                       # 40 idle + 90 > 100: idle ones go, least recently used first
    assert g == 90 and closed == ["a1", "b1", "a2"] and srv._used == 90
    srv._release(g)
    srv.close()
    assert sorted(closed) == ["a1", "a2", "b1"] and srv.cached_contexts() == 0 and srv._used == 0


def test_request_stream_with_repeated_designs():
    from turbomodal_gb300.meshgen import TITANIUM
    from turbomodal_gb300.serve import request_stream, sector_key

    reqs = request_stream(8, seed=11, max_nodes=6000, distinct_sectors=2)
    assert len({sector_key(r.mesh, TITANIUM) for r in reqs}) <= 2


@pytest.mark.gpu
def test_reused_contexts_give_fresh_results():
    """Requests on repeated designs reuse a kept context (its sector matrices, operator patterns
    and symbolic analyses); each result equals the request solved alone on a fresh solver."""
    from turbomodal_gb300.serve import ModalServer, request_stream
    from turbomodal_gb300.solver import CyclicSymmetrySolver

    reqs = request_stream(6, seed=7, rate_hz=50.0, min_nodes=2000, max_nodes=9000, distinct_sectors=2)
    srv = ModalServer(budget_bytes=24 << 30, max_inflight=2)
    done = srv.serve(reqs)
    srv.close()
    assert all(not c.error for c in done), [c.error for c in done]
    assert sum(c.reused for c in done) >= 1
    for r, c in zip(sorted(reqs, key=lambda r: r.rid), done):
        s = CyclicSymmetrySolver(r.mesh, r.material, precision=r.precision)
        alone = {x.harmonic_index: x for x in s.solve_at_rpm(r.rpm, r.num_modes, r.harmonics, precision=r.precision)}
        s.close()
        got = {x.harmonic_index: x for x in c.results}
        assert sorted(alone) == sorted(got)
        for k, a in alone.items():
            np.testing.assert_allclose(got[k].frequencies, a.frequencies, rtol=1e-8)


class _FakeSolver:
    made: list = []
    closed: list = []

    def __init__(self):
        self.id = len(_FakeSolver.made)
        _FakeSolver.made.append(self)
        self.calls = []

    def set_memory_budget(self, n):
        pass

    def prepare(self, rpm):
        pass

    def device_bytes(self):
        return 5000, 5000

    def symbolic_stats(self, kind=0):
        return {"n": 100.0, "l_entries": 1e3, "u_entries": 1e3, "lower_entries": 500.0}

    def solve_rpm_sweep(self, rpms, num_modes, ks, precision=None):
        from turbomodal_gb300.solver import ModalResult

        self.calls.append((list(rpms), num_modes, list(ks)))
        if any(r < 0 for r in rpms):
            raise RuntimeError("planted failure")
        return [[ModalResult(k, r, np.arange(1.0, num_modes + 1.0) * (k + 1), np.zeros((3, num_modes), np.complex128),
                             np.zeros(num_modes, np.int32)) for k in ks] for r in rpms]

    def close(self):
        _FakeSolver.closed.append(self.id)


def test_failed_request_context_is_not_kept():
    """A request that fails mid-solve is reported and its context closed instead of cached; the next
    request on the same sector gets a fresh context, a successful one is kept and reused, and every
    reserved byte is returned once the pool is closed."""
    from turbomodal_gb300.meshgen import TITANIUM, sector_mesh
    from turbomodal_gb300.serve import ModalServer, Request

    _FakeSolver.made, _FakeSolver.closed = [], []
    mesh = sector_mesh(4, 3, 1, num_sectors=24, seed=1)
    srv = ModalServer(budget_bytes=1 << 40, max_inflight=1, solver_factory=lambda m, mat, p: _FakeSolver())
    (bad,) = srv._run([Request(0, mesh, TITANIUM, -1.0, 5, [1])], 0.0)
    assert bad.error.startswith("RuntimeError") and _FakeSolver.closed == [0] and srv.cached_contexts() == 0
    assert srv._used == 0
    (ok,) = srv._run([Request(1, mesh, TITANIUM, 1000.0, 5, [1])], 0.0)
    assert not ok.error and not ok.reused and srv.cached_contexts() == 1 and srv._used == 5000
    (again,) = srv._run([Request(2, mesh, TITANIUM, 2000.0, 5, [1])], 0.0)
    assert not again.error and again.reused and len(_FakeSolver.made) == 2
    srv.close()
    assert sorted(_FakeSolver.closed) == [0, 1] and srv._used == 0


def test_same_sector_requests_are_batched():
    """Queued requests on one sector run as one batched sweep with the union of their harmonics
    and the largest mode count; each request gets back its own harmonics and its own number of
    modes, in its own speed's slot."""
    from turbomodal_gb300.meshgen import TITANIUM, sector_mesh
    from turbomodal_gb300.serve import ModalServer, Request

    _FakeSolver.made, _FakeSolver.closed = [], []
    a = sector_mesh(4, 3, 1, num_sectors=24, seed=1)
    b = sector_mesh(5, 3, 1, num_sectors=24, seed=2)
    reqs = [Request(0, a, TITANIUM, 1000.0, 4, [1, 3]), Request(1, b, TITANIUM, 1500.0, 5, [2]),
            Request(2, a, TITANIUM, 2000.0, 6, [3, 7]), Request(3, a, TITANIUM, 3000.0, 2, [])]
    srv = ModalServer(budget_bytes=1 << 40, max_inflight=1, solver_factory=lambda m, mat, p: _FakeSolver())
    done = srv.serve(reqs)
    srv.close()
    assert all(not c.error for c in done)
    calls = [c for s in _FakeSolver.made for c in s.calls]
    batched = [c for c in calls if len(c[0]) > 1]
    assert batched and batched[0][1] == 6 and batched[0][2] == list(range(13))   # union with k = 0..12
    assert [r.harmonic_index for r in done[0].results] == [1, 3]
    assert [r.harmonic_index for r in done[3].results] == list(range(13))
    for c, r in zip(done, reqs):
        assert all(len(x.frequencies) == r.num_modes and x.rpm == r.rpm for x in c.results)
        np.testing.assert_array_equal(c.results[0].frequencies,
                                      np.arange(1.0, r.num_modes + 1.0) * (c.results[0].harmonic_index + 1))
    assert done[0].batched == 3 and done[1].batched == 1


def test_batch_grants_cannot_deadlock():
    """Two requests that hold set-up reservations and then ask for their factorisation batches
    (each wanting the whole rest of the budget) both proceed: a batch grant takes what is free
    once one problem's worth is, and the engine sizes its batches to the grant."""
    from turbomodal_gb300.serve import ModalServer

    srv = ModalServer(budget_bytes=100)
    a_setup, b_setup = srv._acquire(20), srv._acquire(20)
    got = {}

    def batch(name, setup):
        g = srv._acquire_flexible(100 - setup, 10)
        got[name] = g
        time.sleep(0.02)
        srv._release(g)

    ts = [threading.Thread(target=batch, args=(n, 20)) for n in ("a", "b")]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=5)
    assert not any(t.is_alive() for t in ts)
    assert sorted(got) == ["a", "b"] and all(10 <= g <= 60 for g in got.values())
    srv._release(a_setup + b_setup)
    assert srv._used == 0


def test_serving_deadline_reports_unstarted_requests():
    from turbomodal_gb300.meshgen import TITANIUM, sector_mesh
    from turbomodal_gb300.serve import ModalServer, Request

    _FakeSolver.made, _FakeSolver.closed = [], []
    a = sector_mesh(4, 3, 1, num_sectors=24, seed=1)
    b = sector_mesh(5, 3, 1, num_sectors=24, seed=2)
    reqs = [Request(0, a, TITANIUM, 1000.0, 4, [1]), Request(1, b, TITANIUM, 1500.0, 5, [2], arrival=0.3)]
    srv = ModalServer(budget_bytes=1 << 40, max_inflight=1, solver_factory=lambda m, mat, p: _FakeSolver())
    done = srv.serve(reqs, deadline_s=0.1)
    srv.close()
    assert not done[0].error and done[1].error.startswith("not started")
