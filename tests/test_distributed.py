"""bench.py's multi-rank plumbing on CPU (gloo, world size 2): barriers and
max/sum reductions over ranks, and the reference arm's rank handling (only rank
0 works and prints)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(world, rank)
    d.barrier()
    mx = d.max(float(rank + 1) * 10)
    sm = d.sum(float(rank + 1))
    d.close()
    q.put((rank, mx, sm))


def test_dist_reductions_gloo_world_2():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 20.0, 3.0), (1, 20.0, 3.0)]


def test_reference_arm_rank1_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_shard_games_covers_and_balances():
    import numpy as np
    import psi
    sizes = psi.batch_sizes(4096, 100, 200000, 1).astype(np.int64) + 1
    for world in (1, 2, 3, 8):
        parts = psi.shard_games(sizes, world)
        assert len(parts) == world
        allk = np.sort(np.concatenate(parts))
        assert np.array_equal(allk, np.arange(len(sizes)))
        loads = [int(sizes[p].sum()) for p in parts]
        # greedy largest-first: no rank exceeds another by more than the largest game
        assert max(loads) - min(loads) <= int(sizes.max())
        again = psi.shard_games(sizes, world)
        assert all(np.array_equal(a, b) for a, b in zip(parts, again))


def _shard_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "parallel-si_gb300"))
    import torch
    import torch.distributed as td
    import psi
    td.init_process_group("gloo")
    sizes = psi.batch_sizes(300, 100, 200000, 5).astype("int64") + 1
    mine = psi.shard_games(sizes, world)[rank]
    lens = [None] * world
    td.all_gather_object(lens, (rank, mine.tolist(), int(sizes[mine].sum())))
    td.destroy_process_group()
    q.put(lens)


def test_shard_games_gloo_world_2_partition():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    outs = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert outs[0] == outs[1]   # every rank sees the same gathered partition
    parts = {r: set(ix) for r, ix, _ in outs[0]}
    assert parts[0].isdisjoint(parts[1]) and len(parts[0] | parts[1]) == 300
