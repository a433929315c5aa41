"""Multi-rank host logic on CPU: the population is split into contiguous pv
blocks over world_size-2 gloo ranks, each rank evaluates its block, and the
gathered flux equals the single-process evaluation bit for bit (the model is
the oracle here: the sharding logic is what is under test).  Also the step
timing reduction (max over ranks) and the barrier."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_pv_block_partitions_the_population():
    from pytransit_gb300.sharding import pv_block
    for npv in (0, 1, 2, 3, 7, 8, 100, 8193):
        for world in (1, 2, 3, 4, 8):
            blocks = [pv_block(npv, r, world) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == npv
            assert all(b[1] == c[0] for b, c in zip(blocks, blocks[1:]))
            sizes = [b[1] - b[0] for b in blocks]
            assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)
    with pytest.raises(ValueError):
        pv_block(10, 2, 2)


def test_shard_parameters_slices_only_per_pv_arguments():
    from pytransit_gb300.sharding import shard_parameters
    npv = 5
    k = np.arange(npv * 2.0).reshape(npv, 2)
    ldc_shared = np.ones((npv, 2))          # [npb=5, ncoef]: shared by all pv, not sliced
    t0 = np.arange(npv * 1.0)
    p = np.full(npv, 3.0)
    out = shard_parameters(1, 3, k, ldc_shared, t0, p, 10.0, np.full(npv, 1.5), 0.0, 0.0)
    assert np.array_equal(out[0], k[1:3]) and out[1].shape == (npv, 2)
    assert np.array_equal(out[2], t0[1:3]) and out[3].shape == (2,) and float(out[4]) == 10.0
    assert out[5].shape == (2,) and float(out[6]) == 0.0
    ldc = np.ones((npv, 3, 2))
    assert shard_parameters(0, 2, k, ldc, t0, p, 10.0, 1.5)[1].shape == (2, 3, 2)


def _population(npv, seed, npb=1):
    rng = np.random.default_rng(seed)
    k = rng.uniform(0.05, 0.15, (npv, npb))
    ldc = np.stack([rng.uniform(0, .6, (npv, npb)), rng.uniform(0, .3, (npv, npb))], -1)
    t0 = rng.normal(0, 1e-3, npv)
    p = rng.uniform(1, 10, npv)
    a = rng.uniform(3, 20, npv)
    inc = np.arccos(rng.uniform(0, .9, npv) / a)
    e = rng.uniform(0, .3, npv)
    w = rng.uniform(0, 2 * np.pi, npv)
    return k, ldc, t0, p, a, inc, e, w


def _worker(rank, world, port, errfile):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    import oracle
    from pytransit_gb300 import sharding
    try:
        dist.init_process_group("gloo", rank=rank, world_size=world)
        time = np.linspace(-0.15, 0.15, 300)
        # light curves, a population that does not divide evenly over the ranks
        m = oracle.OracleRoadRunner('quadratic')
        m.set_data(time, nsamples=[3], exptimes=[0.01])
        prm = _population(7, 11)
        got = sharding.evaluate_sharded(m, *prm)
        want = m.evaluate(*prm)
        assert got.shape == want.shape == (7, 300), got.shape
        assert np.array_equal(got, want)
        block, (s0, s1) = sharding.evaluate_sharded(m, *prm, gather=False)
        assert (s0, s1) == sharding.pv_block(7, rank, world)
        assert np.array_equal(block, want[s0:s1])
        # one parameter vector: the second rank's block is empty
        prm1 = tuple(x[:1] for x in prm)
        got1 = sharding.evaluate_sharded(m, *prm1)
        assert got1.shape == (300,) and np.array_equal(got1, m.evaluate(*prm1))
        # transmission spectroscopy: [npv, npb, npt] blocks
        ts = oracle.OracleRoadRunner('quadratic', ts=True)
        ts.set_data(time, nsamples=[3], exptimes=[0.01])
        prm_ts = _population(5, 12, npb=4)
        got_ts = sharding.evaluate_sharded(ts, *prm_ts)
        want_ts = ts.evaluate(*prm_ts)
        assert got_ts.shape == want_ts.shape == (5, 4, 300) and np.array_equal(got_ts, want_ts)
        # the step timing reduction and the barrier
        assert sharding.max_over_ranks(1.0 + rank) == float(world)
        sharding.barrier()
        dist.destroy_process_group()
    except BaseException as ex:  # reported to the parent through the file
        with open(errfile, "a") as f:
            f.write(f"rank {rank}: {type(ex).__name__}: {ex}\n")
        raise


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_evaluate_sharded_gloo_world2(tmp_path):
    import torch.multiprocessing as mp
    pytest.importorskip("torch.distributed")
    errfile = str(tmp_path / "err.txt")
    world = 2
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, errfile)) for r in range(world)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(timeout=180)
    for pr in procs:
        if pr.is_alive():
            pr.kill()
            pr.join()
    err = open(errfile).read() if os.path.exists(errfile) else ""
    assert all(pr.exitcode == 0 for pr in procs), err or [pr.exitcode for pr in procs]


def test_without_process_group_is_plain_evaluate():
    import oracle
    from pytransit_gb300 import sharding
    m = oracle.OracleRoadRunner('quadratic')
    m.set_data(np.linspace(-0.1, 0.1, 50))
    prm = _population(3, 5)
    assert np.array_equal(sharding.evaluate_sharded(m, *prm), m.evaluate(*prm))
    assert sharding.max_over_ranks(2.5) == 2.5
    sharding.barrier()
