"""The handle's cache of counted blocks.

A handle keeps the block it counted last and up to 16 earlier ones; a block
is reused only when its L, spin, full, length and every configuration record
match (compared on the device), so cycling through the symmetry blocks skips
their planning and count passes without ever returning a stale block.
"""
import numpy as np
import pytest

from cases import CASES, assert_csr_close, blocks, oracle_reference

pytestmark = pytest.mark.gpu


def _handle(bs2e):
    c = CASES["small2"]
    ref = oracle_reference("small2")
    h = bs2e.Bs2e(ref["knots"], c["k"], c["q"], c["max_k"])
    h.slater()
    h.rk()
    h.set_one_body(ref["H1p"], ref["S"])
    return h


def _oracle(oracle, cf, L, spin, full=True):
    c = CASES["small2"]
    ref = oracle_reference("small2")
    return oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"], ref["H1p"],
                                  ref["S"], full, spin)


def test_cycling_blocks_and_modified_list(bs2e, oracle):
    bl = blocks(bs2e, "small2")
    want = {}
    with _handle(bs2e) as h:
        for rnd in range(3):
            for (L, M, par, spin, cf) in bl:
                key = (L, spin)
                if key not in want:
                    want[key] = _oracle(oracle, cf, L, spin)
                H, S = h.block(cf, L, True, spin)
                assert_csr_close(H, want[key][0], 1e-12)
                assert_csr_close(S, want[key][1], 1e-12, with_scale=False)
        # same identity (L, spin, full, length) but another list: the channel
        # segments in reverse order (a valid list whose CSR columns differ)
        (L, M, par, spin, cf) = bl[1]
        ch = cf["l1"] * 100 + cf["l2"]
        starts = [0] + [int(i) for i in np.flatnonzero(np.diff(ch)) + 1] + [cf.size]
        segs = [cf[a:b] for a, b in zip(starts[:-1], starts[1:])]
        cf2 = np.concatenate(segs[::-1])
        assert cf2.size == cf.size and len(segs) > 1
        H2, S2 = h.block(cf2, L, True, spin)
        Hr2, Sr2 = _oracle(oracle, cf2, L, spin)
        assert_csr_close(H2, Hr2, 1e-12)
        assert_csr_close(S2, Sr2, 1e-12, with_scale=False)
        H, S = h.block(cf, L, True, spin)
        assert_csr_close(H, want[(L, spin)][0], 1e-12)
