"""Multi-rank host logic on CPU (gloo, world_size 2): files are size-balanced
across ranks with no data-path exchange; gathering per-rank results in input
order reproduces the single-process digests.  Digests here come from the
oracle (the GPU path per rank is the single-GPU path, tested elsewhere)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from sdhash_gb300 import shard, synth


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, sizes, q):
    import torch.distributed as dist

    from oracle import Oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    O = Oracle()
    mine = shard.shard_sizes(sizes, world)[rank]
    part = []
    for i in mine:
        data = synth.mixture_bytes(77, i, int(sizes[i])).tobytes()
        d = O.digest(f"f{i}", data, 0)
        part.append((i, d.to_string() if d else None))
    gathered = [None] * world
    dist.all_gather_object(gathered, part)
    if rank == 0:
        q.put(shard.merge_in_order(gathered, len(sizes)))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_balance_and_cover():
    sizes = [int(s) for s in synth.log_uniform_sizes(5, 500, 4096, 64 << 20)]
    for world in (1, 2, 3, 8):
        parts = shard.shard_sizes(sizes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)


def test_merge_rejects_duplicates_and_gaps():
    with pytest.raises(ValueError):
        shard.merge_in_order([[(0, "a")], [(0, "b")]], 1)
    with pytest.raises(ValueError):
        shard.merge_in_order([[(0, "a")]], 2)


def test_two_rank_gloo_digests_equal_single_process():
    from oracle import Oracle, build_oracle
    build_oracle()
    sizes = [int(s) for s in synth.log_uniform_sizes(6, 12, 600, 400000)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    O = Oracle()
    single = []
    for i, n in enumerate(sizes):
        d = O.digest(f"f{i}", synth.mixture_bytes(77, i, n).tobytes(), 0)
        single.append(d.to_string() if d else None)
    assert merged == single
