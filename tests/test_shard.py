"""Query sharding over ranks: ranges, and the gather of per-rank results on
rank 0 over a two-rank gloo group (CPU)."""
import os
import socket

import pytest

from pplacer_gb300.shard import place_sharded, shard_range


def test_shard_ranges_cover_every_query_once():
    for n in (0, 1, 7, 10, 1001):
        for world in (1, 2, 3, 8):
            got = [shard_range(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [hi - lo for lo, hi in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(5, 2, 2)


def _fake_place(seqs):
    # a deterministic stand-in for Engine.place: one placement per query
    return [[(len(s), -float(sum(map(ord, s))), 1.0, 0.1, 0.2)] for s in seqs], [len(s) % 3 for s in seqs]


def _rank_main(rank, world, port, seqs, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = place_sharded(_fake_place, seqs, rank, world, group=dist.group.WORLD)
        if rank == 0:
            out.put(got)
        else:
            assert got is None
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_gather_two_ranks_gloo():
    import torch.multiprocessing as mp
    seqs = ["ACGT" * (i % 5 + 1) + "-" * i for i in range(11)]
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, seqs, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = out.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    want = _fake_place(seqs)
    assert got[0] == want[0] and got[1] == want[1]


def test_single_process():
    seqs = ["AC", "GTT", "A"]
    assert place_sharded(_fake_place, seqs, 0, 1) == _fake_place(seqs)
