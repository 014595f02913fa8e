"""Sharded runs (ramp_gb300.shard) on two CPU ranks over gloo.

Each rank traces its slice of every chunk with the oracle and the ranks sum
their tallies with one all-reduce, the exchange step of a multi-GPU run;
the sum must equal a single run of all histories within the reordering
error of float additions.  The slices follow the product's rule (the first
chunk's slice, clipped), so carried RNG counters stay with their index in
a multi-chunk run whose last chunk is short.
"""
import os
import random
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from ramp_gb300.shard import chunk_slices, shard_slice

N, CHUNK = 50_001, 20_000


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        import ramp_gb300 as m
        from ramp_gb300 import instruments as I, shard
        ci = m.Instrument(I.path("small_chain.json"), "cpu", **I.small_chain_kwargs())
        random.seed(1234)
        oracle.run(ci, N, chunk=CHUNK, shard=(rank, world), threads=2)
        shard.allreduce_tallies(ci)
        g = torch.full((22,), float(rank + 1), dtype=torch.float64)
        shard.allreduce_gradient(g)
        if rank == 0:
            np.savez(out, grad=g.numpy(), *[t.numpy() for t in ci.tallies()])
    finally:
        dist.destroy_process_group()


def test_chunk_slices_cover_every_index_once():
    for n, c, world in [(50_001, 20_000, 2), (10, 3, 4), (7, 100, 3), (1, 1, 2)]:
        per_chunk = {}
        for r in range(world):
            for k, (torun, lo, cnt) in enumerate(chunk_slices(n, c, r, world)):
                per_chunk.setdefault(k, (torun, []))[1].extend(range(lo, lo + cnt))
        assert sum(t for t, _ in per_chunk.values()) == n
        for torun, idx in per_chunk.values():
            assert sorted(idx) == list(range(torun))
    # a rank keeps the same global indices in every chunk
    assert {lo for _, lo, _ in chunk_slices(50_001, 20_000, 1, 2)} == {10_000}
    with pytest.raises(ValueError):
        shard_slice(10, 2, 2)


def test_two_gloo_ranks_sum_to_a_single_run(tmp_path):
    import oracle
    import ramp_gb300 as m
    from ramp_gb300 import instruments as I
    from helpers import tallies_close

    oracle.lib()                      # built before the ranks start
    out = str(tmp_path / "rank0.npz")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True,
                       start_method="spawn")
    ref = m.Instrument(I.path("small_chain.json"), "cpu", **I.small_chain_kwargs())
    random.seed(1234)
    oracle.run(ref, N, chunk=CHUNK, threads=2)
    got = np.load(out)
    assert np.array_equal(got["grad"], np.full(22, 3.0))

    class Summed:
        def tallies(self):
            return [torch.from_numpy(got["arr_%d" % k]) for k in range(len(ref.tallies()))]

    tallies_close(Summed(), ref)
    assert float(ref.tallies()[0].sum()) > 0
