"""Multi-rank host logic on CPU (gloo, world size 2).

A self-join shards by probe ranges: every rank holds the whole collection and
joins the probes of its range (sqrt split, later probes have longer candidate
windows); ranks exchange nothing on the data path, and only the per-rank pair
lists are gathered at the end.  Here each rank computes its shard with the CPU
oracle (the GPU computes the same shard through `probe_range`, tested in
test_gpu_parity.py::test_probe_ranges_shard_a_join); the test checks that the
shards cover the join exactly once and that the gathered result is the
single-process result."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _worker(rank, world, port, out_q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    import oracle
    from hyset_gb300 import synth

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    c = synth.generate(synth.C2, n_sets=6000, seed=77)
    lo, hi = bench.shard(c.n, world, rank)
    pairs = oracle.join(c.tokens, c.starts, c.sizes, 0.7, probe_range=(lo, hi - 1), index_range=(0, hi - 1)) \
        if hi > lo else np.zeros((0, 2), np.uint32)
    n = torch.tensor([len(pairs)], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n)
    mx = int(max(s.item() for s in sizes))
    buf = torch.zeros((mx, 2), dtype=torch.int64)
    buf[:len(pairs)] = torch.from_numpy(pairs.astype(np.int64))
    bufs = [torch.zeros((mx, 2), dtype=torch.int64) for _ in range(world)]
    dist.all_gather(bufs, buf)
    if rank == 0:
        got = set()
        for s, b in zip(sizes, bufs):
            got |= {tuple(x) for x in b[:int(s.item())].tolist()}
        total = sum(int(s.item()) for s in sizes)
        exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.7))
        out_q.put((got == exp, total == len(exp), [bench.shard(c.n, world, r) for r in range(world)]))
    dist.barrier()
    dist.destroy_process_group()


def test_probe_shards_gather_to_the_whole_join():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    same, exact_count, shards = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert same and exact_count
    assert shards[0][0] == 0 and shards[0][1] == shards[1][0] and shards[1][1] == 6000


def test_shard_split_covers_every_probe_once():
    import bench
    for n in (1, 7, 1000, 1_000_000):
        for ws in (1, 2, 3, 8):
            pts = [bench.shard(n, ws, r) for r in range(ws)]
            assert pts[0][0] == 0 and pts[-1][1] == n
            assert all(pts[i][1] == pts[i + 1][0] for i in range(ws - 1))
