"""Sharding a run's histories across ranks (one process per GPU).

Histories are independent and keyed by their global index within a chunk
(mcramp/include/rand.h:4-21 keys the stream by work-item id), so a chunk
can be cut into contiguous slices, one per rank, with no exchange while
tracing.  Each rank keeps private tallies; the one exchange step is a sum
of the tallies (and, for gradients, of dL/dtheta) across ranks.

Multi-chunk runs carry each index's RNG counter from one chunk to the next
(the reference's neutron buffer persists across chunks, mcramp.py:442-455).
So that a rank's carry stays with the same global indices, every chunk is
cut with the slice of the first (full-size) chunk, clipped to the chunk's
size: a short last chunk leaves the higher ranks less (or no) work, and the
sum over ranks equals a single-device run.
"""
import torch


def shard_slice(n, rank, world):
    """Contiguous slice [lo, lo + count) of n indices for this rank."""
    if not (0 <= rank < world):
        raise ValueError("shard must be (rank, world) with 0 <= rank < world")
    lo = n * rank // world
    hi = n * (rank + 1) // world
    return lo, hi - lo


def chunk_slices(N, buf_max, rank, world):
    """Per chunk of an N-history run with chunks of buf_max: (chunk size,
    first global index of this rank, histories of this rank)."""
    frame = min(N, buf_max)
    lo, cnt = shard_slice(frame, rank, world)
    out = []
    remaining = N
    while remaining > 0:
        torun = buf_max if remaining > buf_max else remaining
        remaining -= torun
        out.append((torun, lo, max(0, min(lo + cnt, torun) - lo)))
    return out


def allreduce_tallies(inst, group=None):
    """Sum every tally of ``inst`` over the ranks of ``group`` (in place)."""
    import torch.distributed as dist
    for t in inst.tallies():
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)


def allreduce_gradient(grad, group=None):
    """Sum a gradient (e.g. DiffChain.gradient) over the ranks, in place."""
    import torch.distributed as dist
    dist.all_reduce(grad, op=dist.ReduceOp.SUM, group=group)
    return grad
