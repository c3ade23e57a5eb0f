"""Served request stream: admission by device-memory budget (host logic, CPU) and, on the GPU,
concurrent requests whose results equal the same requests solved alone.

Tolerance: frequencies of a request in the mix within 1e-9 relative of the request alone (the
per-problem arithmetic does not depend on what else runs; 1e-6 is the parity bar)."""

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
            np.testing.assert_allclose(mixed[k].frequencies, a.frequencies, rtol=1e-9)


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
    """Idle contexts are handed to later requests on the same sector; beyond max_cached the least
    recently used are closed."""
    from turbomodal_gb300.serve import ModalServer

    made, closed = [], []

    class Fake:
        def __init__(self, tag):
            self.tag = tag

        def close(self):
            closed.append(self.tag)

    def factory(mesh, material, precision):
        made.append(mesh)
        return Fake(f"{mesh}-{len(made)}")

    srv = ModalServer(budget_bytes=1, max_cached=2, solver_factory=factory)
    s1, r1 = srv._checkout("A", "A", None, "mixed")
    assert not r1 and made == ["A"]
    srv._checkin("A", s1)
    s2, r2 = srv._checkout("A", "A", None, "mixed")
    assert r2 and s2 is s1 and made == ["A"]
    s3, r3 = srv._checkout("A", "A", None, "mixed")          # the only idle one is in use
    assert not r3 and made == ["A", "A"]
    srv._checkin("A", s2)
    srv._checkin("A", s3)
    b1, _ = srv._checkout("B", "B", None, "mixed")
    srv._checkin("B", b1)                                     # 3 idle > 2: the oldest A goes
    assert closed == [s2.tag] and srv.cached_contexts() == 2
    srv.close()
    assert sorted(closed) == sorted([s2.tag, s3.tag, b1.tag]) and srv.cached_contexts() == 0


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
            np.testing.assert_allclose(got[k].frequencies, a.frequencies, rtol=1e-9)


def test_failed_request_context_is_not_kept():
    """A request that fails mid-solve is reported and its context closed instead of cached; the next
    request on the same sector gets a fresh context, a successful one is kept and reused."""
    from turbomodal_gb300.meshgen import TITANIUM, sector_mesh
    from turbomodal_gb300.serve import ModalServer, Request

    closed, made = [], []

    class FakeSolver:
        def __init__(self):
            self.id = len(made)
            made.append(self)

        def set_memory_budget(self, n):
            pass

        def prepare(self, rpm):
            pass

        def symbolic_stats(self, kind=0):
            return {"n": 100.0, "l_entries": 1e3, "u_entries": 1e3, "lower_entries": 500.0}

        def solve_at_rpm(self, rpm, num_modes, ks, precision=None):
            if rpm < 0:
                raise RuntimeError("planted failure")
            return []

        def close(self):
            closed.append(self.id)

    mesh = sector_mesh(4, 3, 1, num_sectors=24, seed=1)
    srv = ModalServer(budget_bytes=1 << 40, max_inflight=1, solver_factory=lambda m, mat, p: FakeSolver())
    bad = srv._run(Request(0, mesh, TITANIUM, -1.0, 5, [1]), 0.0)
    assert bad.error.startswith("RuntimeError") and closed == [0] and srv.cached_contexts() == 0
    ok = srv._run(Request(1, mesh, TITANIUM, 1000.0, 5, [1]), 0.0)
    assert not ok.error and not ok.reused and srv.cached_contexts() == 1
    again = srv._run(Request(2, mesh, TITANIUM, 2000.0, 5, [1]), 0.0)
    assert not again.error and again.reused and len(made) == 2
    assert srv._used == 0
    srv.close()
    assert sorted(closed) == [0, 1]
