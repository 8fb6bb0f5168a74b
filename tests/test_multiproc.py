"""The N > 1 bench path on CPU: two gloo ranks shard the batch by seed and
take the slowest rank's time; the reference arm runs on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, _ = bench.dist_setup(world)
    base = bench.shard_base(r, 4096)
    t = bench.max_over_ranks(10.0 + 5.0 * r, w, device="cpu")
    # a throttled region on one rank makes every rank measure again
    again = (bench.any_rank(r == 1, w, device="cpu"), bench.any_rank(False, w, device="cpu"))
    # every rank's seeds are disjoint from the others'
    seeds = set(range(base, base + 4096))
    gathered = [None] * w
    dist.all_gather_object(gathered, sorted(seeds)[:1] + sorted(seeds)[-1:])
    dist.destroy_process_group()
    q.put((r, w, base, t, gathered, again))


def test_two_gloo_ranks_shard_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, b0, t0, g0, a0), (r1, w1, b1, t1, g1, a1) = out
    assert a0 == a1 == (True, False)
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert b1 - b0 == 4096                 # disjoint seed ranges
    assert t0 == t1 == 15.0                # the job's time is the slowest rank's
    (lo0, hi0), (lo1, hi1) = g0
    assert hi0 < lo1


def test_reference_arm_runs_on_rank0_only(monkeypatch, capsys):
    import argparse

    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(gpus=2, steps=1, warmup=0, count=8)
    bench.run_reference(args)          # returns before any work on rank 1
    assert capsys.readouterr().out == ""


def test_clock_screen():
    import bench
    assert bench.clocks_ok({"sm_mhz": 2070, "sm_max_mhz": 2070, "reasons": []})
    assert bench.clocks_ok({"sm_mhz": 1700, "sm_max_mhz": 2070, "reasons": ["sw_power_cap"]})
    for r in bench.THROTTLE_REASONS:
        assert not bench.clocks_ok({"sm_mhz": 2070, "sm_max_mhz": 2070, "reasons": [r]})
    assert not bench.clocks_ok({"sm_mhz": 1200, "sm_max_mhz": 2070, "reasons": []})  # clock lock


def test_clock_sample_parsing():
    import bench
    c = bench.Clocks(0)
    c.lines = ["0, 2070, 2070, 900.1, Not Active, Not Active, Not Active, Not Active, Not Active",
               "0, 2055, 2070, 1390.0, Active, Not Active, Not Active, Not Active, Active",
               "garbage"]
    s = c.summary()
    assert s["sm_max_mhz"] == 2070 and s["samples"] == 2 and s["reasons"] == ["sw_power_cap"]
    assert bench.clocks_ok(s)
    c.lines = ["0, 1100, 2070, 500.0, Active, Active, Not Active, Not Active, Not Active"]
    s = c.summary()
    assert s["reasons"] == ["hw_slowdown"] and not bench.clocks_ok(s)


def _shard_worker(rank, world, port, q):
    # Each rank rounds its part of one batch with the oracle (the CPU worker
    # of this test); rank 0 gathers through host memory (gloo).
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import pyoracle as O
    from tensor_train_gb300 import shard
    tts = [O.random_uneven(1000 + i, 8, 12, 4, 16) for i in range(24)]
    mine = shard.my_part(tts, rank, world)
    ys = shard.round_batch_distributed(tts, worker=lambda part: [O.round(t, 1e-8) for t in part])
    dist.destroy_process_group()
    q.put((rank, mine, ys))


def test_two_gloo_ranks_round_one_batch():
    import numpy as np
    from oracle import pyoracle as O
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in procs), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, mine0, ys0), (_, mine1, ys1) = out
    assert ys1 is None and ys0 is not None
    # the parts cover the batch once, and both ranks did work
    assert sorted(mine0 + mine1) == list(range(24)) and mine0 and mine1
    # the gathered result equals the single-rank result bit for bit, in order
    tts = [O.random_uneven(1000 + i, 8, 12, 4, 16) for i in range(24)]
    single = [O.round(t, 1e-8) for t in tts]
    for a, b in zip(ys0, single):
        assert len(a) == len(b) and all(np.array_equal(x, y) for x, y in zip(a, b))


def test_shard_plan_balances_by_cost(ttg):
    # Longest estimated cost first to the least-loaded part: deterministic,
    # every TT placed once, loads within the largest single cost.
    import numpy as np
    from oracle import pyoracle as O
    from tensor_train_gb300.flops import round_flops
    tts = [O.random_uneven(1000 + i) for i in range(64)]
    part_of, cost = ttg.shard_plan(tts, 3)
    assert np.array_equal(part_of, ttg.shard_plan(tts, 3)[0])
    assert set(part_of.tolist()) == {0, 1, 2}
    for t, c in zip(tts, cost):
        modes = [x.shape[1] for x in t]
        r = [t[0].shape[0]] + [x.shape[-1] for x in t]
        assert abs(c - round_flops(modes, r, r)) <= 1e-9 * c
    loads = [cost[part_of == p].sum() for p in range(3)]
    assert max(loads) - min(loads) <= cost.max()
    assert np.array_equal(ttg.shard_plan(tts, 1)[0], np.zeros(64, np.int32))
