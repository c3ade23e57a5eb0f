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


def test_reference_arm_prints_its_line(monkeypatch, capsys):
    """bench.py --impl reference (the reference's CPU algorithm sampled on the host cores) prints
    one JSON line with the contract's keys; it needs no GPU.  The sampler runs here on the
    config-0 sector to keep the CPU suite short (the bench uses the config-1 sector)."""
    import json

    import bench
    from turbomodal_gb300.meshgen import config_mesh

    small = config_mesh(0)

    class Small(bench.ReferenceSample):
        def __init__(self, threads=None, target_window_s=4.0, planned_samples=0, mesh=None):
            super().__init__(threads=2, target_window_s=0.05, planned_samples=planned_samples, mesh=small)

    monkeypatch.setattr(bench, "ReferenceSample", Small)
    args = bench.argparse.Namespace(gpus=1, steps=2, warmup=1)
    bench.run_reference(args, 1, 0, None)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 2
    assert line["steps"] == 2 and line["ms_per_step"] > 0 and line["config"]["workload"]


def test_window_samples_add_up_to_the_whole_factorisation():
    """The reference sampler's estimate of one factorisation (W equal-work row windows of the
    up-looking LDL^H, each timed alone) against the same loop run over all rows at once, on the
    config-0 harmonic operator: within 30 % (the windows start with cold caches), and the loop
    work the symbolic pass counts equals sum_j c_j (c_j + 1) / 2 over the column counts."""
    import scipy.sparse as sp

    from oracle import orc
    from turbomodal_gb300.meshgen import TITANIUM, config_mesh

    om = orc.OracleModel(config_mesh(0), TITANIUM)
    om.prepare(0.0)
    A = (om.matrix("Kk", k=1) - om.matrix("Mk", k=1)).tocsc()
    lw = orc.LdlWindows(A)
    _, _, cc = orc.ldl_symbolic(sp.tril(A).tocsc())
    assert lw.total_work == int(np.sum(cc.astype(np.int64) * (cc + 1) // 2))
    cum = lw.cumwork()
    assert cum[0] == 0 and cum[-1] == lw.total_work and np.all(np.diff(cum) >= 0)
    full = min(lw.run([0], [0], [lw.n], solve=False)[0][0] for _ in range(3))
    W = 16
    bnd = np.searchsorted(cum, np.linspace(0, cum[-1], W + 1))
    bnd[0], bnd[-1] = 0, lw.n
    parts = [min(lw.run([0], [bnd[j]], [bnd[j + 1]], solve=False)[0][0] for _ in range(3)) for j in range(W)]
    assert 0.7 * full <= sum(parts) <= 1.3 * full, (full, sum(parts))
