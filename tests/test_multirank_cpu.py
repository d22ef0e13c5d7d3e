"""Multi-rank host logic on CPU (two gloo ranks), through the library.

A multi-GPU basis setup splits the symmetry blocks into n1 bands
(bs2e_band_plan: bands that fit a buffer, each owned by one rank, every rank
computing the same plan without communicating), each rank assembles the rows
of its bands (bs2e_band_rows gives them; on a GPU bs2e_block_fill_band fills
them), and the rank that needs whole blocks gathers the band CSRs and joins
them (bs2e_band_merge), as CS_from_block_diag joins blocks
(src/tools/block_tools.f90:289-348).  The path has no exchange step: the
only collective is the final gather.

Here the ranks have no GPU, so each band's CSR is cut from the oracle's
whole block (standing in for the device fill); what runs is the library's
planning, row lists and join, and the joined blocks must equal the oracle's
bit for bit, with every band owned by exactly one rank.
"""
import os
import socket

import numpy as np

from cases import CASES, blocks, oracle_reference


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _per_n1(cf, H, S, n_b):
    """(rows, nnz_H, nnz_S) per n1 of a whole block's CSR (what
    bs2e_block_band_count returns on a GPU)."""
    lenH = np.diff(H["index_ptr"])
    lenS = np.diff(S["index_ptr"])
    out = np.zeros((n_b, 3), dtype=np.int64)
    np.add.at(out[:, 0], cf["n1"] - 1, 1)
    np.add.at(out[:, 1], cf["n1"] - 1, lenH)
    np.add.at(out[:, 2], cf["n1"] - 1, lenS)
    return out


def _cut(M, rows1):
    """CSR of 1-based block rows `rows1` of a whole-block CSR."""
    ptr = M["index_ptr"]
    r = rows1 - 1
    lens = ptr[r + 1] - ptr[r]
    sel = np.concatenate([np.arange(ptr[i] - 1, ptr[i + 1] - 1) for i in r]) if r.size \
        else np.zeros(0, np.int64)
    return dict(index_ptr=np.concatenate([[1], 1 + np.cumsum(lens)]).astype(np.int64),
                indices=M["indices"][sel], data=M["data"][sel])


def _whole_blocks(O, pkg):
    c = CASES["small2"]
    ref = oracle_reference("small2")
    out = []
    for (L, M, par, spin, cf) in blocks(pkg, "small2"):
        H, S = O.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"], ref["H1p"],
                                 ref["S"], True, spin)
        out.append((cf, H, S))
    return out


# a buffer that splits every small2 block into several bands (one n1 of the
# largest block needs 9.6 MB; whole blocks need 40-205 MB)
MAX_BYTES = 24 << 20


def _worker(rank, world, port, out_q):
    try:
        _work(rank, world, port, out_q)
    except BaseException:
        import traceback
        out_q.put(("error", rank, traceback.format_exc()))
        raise


def _work(rank, world, port, out_q):
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
    n_b = CASES["small2"]["n_b"]
    whole = _whole_blocks(O, pkg)
    plan = pkg.band_plan([_per_n1(cf, H, S, n_b) for (cf, H, S) in whole], MAX_BYTES, world)
    mine = []
    for (b, a, m, owner, nbytes) in plan:
        if owner != rank:
            continue
        cf, H, S = whole[b]
        rows = pkg.band_rows(cf, a, m)
        mine.append((int(b), rows, _cut(H, rows), _cut(S, rows)))
    gathered = [None] * world
    dist.all_gather_object(gathered, (plan, mine))
    dist.destroy_process_group()
    if rank == 0:
        out_q.put(gathered)


def test_two_rank_bands_join_to_the_oracle_blocks(bs2e, oracle):
    import torch.multiprocessing as mp
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=600)
    assert not (isinstance(gathered, tuple) and gathered[0] == "error"), gathered
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    plans = [g[0] for g in gathered]
    assert all(np.array_equal(plans[0], p) for p in plans)  # same plan on every rank
    plan = plans[0]
    assert set(plan[:, 3].tolist()) == {0, 1}  # both ranks own bands
    assert len(plan) > len(_whole_blocks(oracle, bs2e))  # some blocks split
    pieces = {}
    for (_, mine) in gathered:
        for (b, rows, H, S) in mine:
            pieces.setdefault(b, []).append((rows, H, S))
    for b, (cf, H, S) in enumerate(_whole_blocks(oracle, bs2e)):
        parts = pieces[b]
        for which, ref in ((1, H), (2, S)):
            got = bs2e.band_merge(cf.size, [dict(rows=p[0], **p[which]) for p in parts])
            for x in ("index_ptr", "indices", "data"):
                np.testing.assert_array_equal(got[x], ref[x])


def test_band_plan_and_rows(bs2e, oracle):
    n_b = CASES["small2"]["n_b"]
    whole = _whole_blocks(oracle, bs2e)
    per = [_per_n1(cf, H, S, n_b) for (cf, H, S) in whole]
    for world in (1, 2, 3, 8):
        plan = bs2e.band_plan(per, MAX_BYTES, world)
        for b, (cf, H, S) in enumerate(whole):
            mine = plan[plan[:, 0] == b]
            # bands of a block tile 1..n_b without gaps (empty n1 ranges aside)
            covered = np.concatenate([np.arange(a, a + m) for (_, a, m, _, _) in mine])
            assert np.all(np.diff(covered) == 1)
            assert set(cf["n1"].tolist()) <= set(covered.tolist())
            rows = np.concatenate([bs2e.band_rows(cf, a, m) for (_, a, m, _, _) in mine])
            np.testing.assert_array_equal(np.sort(rows), np.arange(1, cf.size + 1))
            assert (mine[:, 4] <= MAX_BYTES).all()
        loads = np.bincount(plan[:, 3], weights=plan[:, 4], minlength=world)
        assert loads.max() - loads.min() <= plan[:, 4].max()
    # a single n1 above the buffer is refused
    import pytest
    with pytest.raises(bs2e.Bs2eError):
        bs2e.band_plan(per, 1024, 1)
    # a join with a row missing or repeated is refused
    cf, H, S = whole[0]
    rows = bs2e.band_rows(cf, 1, n_b)
    part = dict(rows=rows[:-1], **_cut(H, rows[:-1]))
    with pytest.raises(bs2e.Bs2eError):
        bs2e.band_merge(cf.size, [part])
    with pytest.raises(bs2e.Bs2eError):
        bs2e.band_merge(cf.size, [part, dict(rows=rows[:2], **_cut(H, rows[:2]))])
