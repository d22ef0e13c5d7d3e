"""The batched radial stage (bs2e_batch_*): a ragged batch of bases, one
persistent kernel per stage, graph-captured after the first run.

Its results must be bit-identical to each handle's own bs2e_slater + bs2e_rk
(both run the same device functions), on every run (the first, tuning run and
the graph replays), for FP64 and mixed handles in one batch.
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

# order, spline count, r_max, GL points, max_k, precision (0 FP64, 1 mixed)
SMALL = [(6, 40, 40.0, 10, 4, 0), (8, 31, 31.0, 12, 9, 1), (7, 55, 55.0, 11, 12, 0),
         (5, 24, 20.0, 7, 3, 1), (6, 47, 47.0, 9, 16, 0), (7, 36, 36.0, 11, 6, 0)]


def test_ragged_problem_list_matches_fixture(bs2e):
    want = json.load(open(os.path.join(HERE, "golden", "ragged_problems.json")))
    assert bs2e.grids.ragged_problems(64, 0) == want
    ks = {p["k"] for p in want}
    assert ks <= {6, 7, 8} and all(100 <= p["n_b"] <= 500 for p in want)
    assert all(4 <= p["max_k"] <= 16 and 0 <= p["l_max"] <= 8 for p in want)


def _make(bs2e, spec):
    k, N, r_max, q, max_k, prec = spec
    t = bs2e.grids.explin_knots(k, N, r_max)
    return bs2e.Bs2e(t, k, q, max_k, precision=prec)


def _store(h):
    return [h.rk_export(kk) for kk in range(h.K1)]


@pytest.mark.gpu
def test_batch_bit_identical_to_per_handle(bs2e):
    ref = []
    for spec in SMALL:
        with _make(bs2e, spec) as h:
            h.slater()
            h.rk()
            ref.append((_store(h), h.primitives()))
    hs = [_make(bs2e, spec) for spec in SMALL]
    try:
        with bs2e.RadialBatch(hs) as b:
            for run in range(3):  # tuning run, then graph replays
                b.run()
                info = b.tuning()
                assert info["graph"] and info["rk_threads"] in (128, 256, 512)
                for h, (R, prim) in zip(hs, ref):
                    got = _store(h)
                    for kk in range(h.K1):
                        np.testing.assert_array_equal(got[kk], R[kk])
                    if run == 0:
                        p = h.primitives()
                        for name in ("r_k", "r_m_k", "r_d_k", "idx4", "idx6"):
                            np.testing.assert_array_equal(p[name], prim[name])
            assert b.tuning()["launches"] >= 4 + 9 + 8
    finally:
        for h in hs:
            h.close()


@pytest.mark.gpu
def test_batch_handles_usable_for_blocks(bs2e, oracle):
    """After the batched radial stage a handle assembles blocks as usual."""
    from cases import CASES, blocks, oracle_reference, assert_csr_close
    c = CASES["small2"]
    ref = oracle_reference("small2")
    h = bs2e.Bs2e(ref["knots"], c["k"], c["q"], c["max_k"])
    other = _make(bs2e, SMALL[2])
    try:
        with bs2e.RadialBatch([other, h]) as b:
            b.run()
        h.set_one_body(ref["H1p"], ref["S"])
        (L, M, par, spin, cf) = [x for x in blocks(bs2e, "small2") if x[0] == 1][0]
        H, S = h.block(cf, L, True, spin)
        Hr, Sr = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"],
                                        ref["H1p"], ref["S"], True, spin)
        assert_csr_close(H, Hr, 1e-12)
    finally:
        h.close()
        other.close()


@pytest.mark.gpu
def test_batch_rejects_duplicates(bs2e):
    h = _make(bs2e, SMALL[0])
    try:
        with pytest.raises(bs2e.Bs2eError):
            bs2e.RadialBatch([h, h])
    finally:
        h.close()
