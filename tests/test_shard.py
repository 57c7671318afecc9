"""Multi-rank field sharding on CPU: two gloo ranks (spawned processes) split a
batch into whole-field blocks, "advance" their own block, and gather the batch;
every rank must end with every field, in order, exactly once."""

import os
import tempfile

import torch
import torch.multiprocessing as mp

from nlse_gb300.shard import field_block, gather_fields


def test_blocks_partition_the_batch():
    for n in (0, 1, 7, 8, 164):
        for world in (1, 2, 3, 8):
            blocks = [field_block(n, r, world) for r in range(world)]
            covered = [i for b in blocks for i in range(b.start, b.stop)]
            assert covered == list(range(n))
            sizes = [b.stop - b.start for b in blocks]
            assert max(sizes) - min(sizes) <= 1


def _rank(rank, world, store_file, n, q):
    import torch.distributed as dist

    # a file rendezvous: no port to race for with other processes
    dist.init_process_group("gloo", init_method=f"file://{store_file}", rank=rank,
                            world_size=world)
    try:
        blk = field_block(n, rank, world)
        fields = torch.arange(n * 6, dtype=torch.float64).reshape(n, 3, 2)
        local = torch.complex(fields[blk], -fields[blk]) * (rank + 1) / (rank + 1)
        full = gather_fields(local.contiguous(), n)
        q.put((rank, blk.start, blk.stop, full.numpy()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_every_field_once():
    n, world = 7, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    store_file = os.path.join(tempfile.mkdtemp(prefix="nlse_gloo_"), "store")
    procs = [ctx.Process(target=_rank, args=(r, world, store_file, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    fields = torch.arange(n * 6, dtype=torch.float64).reshape(n, 3, 2)
    expect = torch.complex(fields, -fields).numpy()
    starts = sorted((r[1], r[2]) for r in results)
    assert starts == [(0, 4), (4, 7)]
    for _, _, _, full in results:
        assert (full == expect).all()
