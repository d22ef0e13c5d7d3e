"""Multi-rank host logic on CPU: symmetry blocks sharded over two gloo ranks
give the same CSR blocks as one process (the path has no exchange step; the
gather is the host-side concatenation CS_from_block_diag does,
src/tools/block_tools.f90:274-348)."""
import os
import socket

import numpy as np
import pytest

from cases import CASES, blocks, oracle_reference


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_q):
    import sys
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    from conftest import load_package
    import oracle as O
    pkg = load_package()
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    c = CASES["small2"]
    ref = oracle_reference("small2")
    bl = blocks(pkg, "small2")
    work = [pkg.basis.block_work(cf.size, len(set(zip(cf["l1"], cf["l2"])))) for (*_, cf) in bl]
    mine = pkg.basis.shard_blocks(work, world, rank)
    res = {}
    for i in mine:
        L, M, par, spin, cf = bl[i]
        H, S = O.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"], ref["H1p"],
                                 ref["S"], True, spin)
        res[i] = (H["index_ptr"], H["indices"], H["data"], S["indices"], S["data"])
    gathered = [None] * world
    dist.all_gather_object(gathered, res)
    dist.destroy_process_group()
    if rank == 0:
        out_q.put(gathered)


def test_two_rank_block_sharding_matches_single_process(bs2e, oracle):
    import torch.multiprocessing as mp
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=600)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    merged = {}
    for part in gathered:
        assert not (set(part) & set(merged))  # each block exactly once
        merged.update(part)
    c = CASES["small2"]
    ref = oracle_reference("small2")
    bl = blocks(bs2e, "small2")
    assert sorted(merged) == list(range(len(bl)))
    for i, (L, M, par, spin, cf) in enumerate(bl):
        H, S = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"], ref["H1p"],
                                      ref["S"], True, spin)
        got = merged[i]
        np.testing.assert_array_equal(got[0], H["index_ptr"])
        np.testing.assert_array_equal(got[1], H["indices"])
        np.testing.assert_array_equal(got[2], H["data"])
        np.testing.assert_array_equal(got[3], S["indices"])
        np.testing.assert_array_equal(got[4], S["data"])


def test_shard_blocks_partition(bs2e):
    work = [5, 9, 9, 3, 7, 1, 8, 2]
    for world in (1, 2, 3, 4, 8):
        parts = [bs2e.basis.shard_blocks(work, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(work)))
        loads = [sum(work[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(work)
