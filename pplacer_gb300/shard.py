"""Query sharding over ranks (one process per GPU).

pplacer's only parallelism is one forked worker per query
(pplacer_src/pplacer_run.ml:628-648): queries are independent and the
reference tree is shared.  Here every rank holds the whole reference
(darr / parr / snodes replicated on its GPU) and places a contiguous range
of the queries; there is no data-path collective, only the host-side
concatenation of the per-query results on rank 0 in query order, as the
reference concatenates its workers' Pquery results before writing
(pplacer_run.ml:552-557).
"""


def shard_range(n, rank, world):
    """The contiguous [lo, hi) of n queries that rank places: sizes differ by
    at most one, lower ranks take the remainder."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def place_sharded(place, seqs, rank, world, group=None):
    """Place this rank's range of seqs with place(list_of_seqs) -> (results,
    statuses) and gather every rank's part on rank 0 over torch.distributed
    (group: the process group; None for a single process).  Rank 0 returns
    (results, statuses) for all queries in order; the other ranks return
    None."""
    lo, hi = shard_range(len(seqs), rank, world)
    res, st = place(seqs[lo:hi])
    part = (lo, list(res), [int(x) for x in st])
    if world == 1:
        return part[1], part[2]
    import torch.distributed as dist
    parts = [None] * world if rank == 0 else None
    dist.gather_object(part, parts, dst=0, group=group)
    if rank != 0:
        return None
    parts.sort(key=lambda p: p[0])
    results, statuses = [], []
    for _, r, s in parts:
        results += r
        statuses += s
    return results, statuses
