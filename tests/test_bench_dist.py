"""The multi-rank bench path on CPU: two gloo ranks shard the speeds without overlap and
combine their timings (max) and eigenpair counts (sum) as bench.py does for N GPUs."""

import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    ws, r, local, pg = bench.dist_setup()
    mine = bench.shard_speeds(bench.RPMS, r, ws)
    t = bench.max_over_ranks(pg, 1.5 + r)
    n = bench.sum_over_ranks(pg, float(len(mine)))
    bench.barrier(pg)
    out.put((r, ws, [float(x) for x in mine], t, n))
    pg.destroy_process_group()


def test_two_ranks_shard_and_reduce():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    import bench

    all_speeds = sorted(res[0][2] + res[1][2])
    assert all_speeds == sorted(float(x) for x in bench.RPMS)
    assert not set(res[0][2]) & set(res[1][2])
    assert all(r[1] == 2 for r in res)
    assert all(r[3] == 2.5 for r in res)                       # max over ranks
    assert all(r[4] == float(len(bench.RPMS)) for r in res)   # sum over ranks


def test_distinct_verified_counts_each_pair_once():
    """Degenerate harmonics return every eigenpair twice (positions 2q, 2q+1); standing ones once."""
    import bench

    class R:
        def __init__(self, k, f, w, conv=True):
            self.harmonic_index, self.frequencies, self.whirl_direction, self.converged = k, np.array(f), np.array(w), conv

    ref = [R(0, [10.0, 20.0, 30.0], [0, 0, 0]), R(1, [11.0, 11.0, 21.0, 21.0, 31.0], [1, -1, 1, -1, 1]),
           R(2, [12.0, 12.0], [1, -1])]
    mix = [R(0, [10.0, 20.0, 30.5], [0, 0, 0]), R(1, [11.0, 11.0, 21.0, 21.0, 31.0], [1, -1, 1, -1, 1]),
           R(2, [12.0, 12.0], [1, -1], conv=False)]
    assert bench.count_distinct_verified(mix, ref) == 2 + 3
    assert bench.count_verified(mix, ref)[0] == 2 + 5


def test_reference_arm_prints_its_line():
    """bench.py --impl reference (the reference's CPU algorithm, timed on the host cores) prints one
    JSON line with the contract's keys; it needs no GPU."""
    import json
    import subprocess
    import sys

    from conftest import ROOT

    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, check=True, capture_output=True, text=True, timeout=600).stdout
    line = json.loads(out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["metric"] and line["unit"] and line["config"]["workload"]
