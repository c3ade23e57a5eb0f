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
