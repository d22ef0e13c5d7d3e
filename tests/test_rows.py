"""Row ranges of a block and the chunked fill into host arrays.

bs2e_block_count_rows / bs2e_block_fill_rows must give exactly the rows
row_first.. of the whole block (the oracle's construct_block over the same row
range, hamiltonian.f90:106-283): bit-exact pointers and columns, values within
1e-12 of the term scale.  Fills into host arrays go through two staging
areas; a small stage_bytes forces many chunks.
"""
import numpy as np
import pytest

from cases import CASES, assert_csr_close, blocks, oracle_reference

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _case_block(bs2e, L, spin):
    return [b for b in blocks(bs2e, "small2") if b[0] == L and b[3] == spin][0]


def _handle(bs2e, precision=0, stage_bytes=0):
    c = CASES["small2"]
    ref = oracle_reference("small2")
    h = bs2e.Bs2e(ref["knots"], c["k"], c["q"], c["max_k"], precision=precision,
                  stage_bytes=stage_bytes)
    h.slater()
    h.rk()
    h.set_one_body(ref["H1p"], ref["S"])
    return h


def _oracle_rows(oracle, cf, L, spin, full, rows):
    c = CASES["small2"]
    ref = oracle_reference("small2")
    return oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"], ref["H1p"],
                                  ref["S"], full, spin, rows=rows)


@pytest.mark.parametrize("L,spin,full", [(1, 0, True), (2, 1, True), (0, 0, False)])
def test_row_ranges_match_oracle(bs2e, oracle, L, spin, full):
    (L, M, par, spin, cf) = _case_block(bs2e, L, spin)
    n = cf.size
    ranges = [(0, 1), (n - 1, n), (n // 3, n // 3 + n // 4), (7, 7), (0, n)]
    with _handle(bs2e) as h:
        for (r0, r1) in ranges:
            H, S = h.block_rows(cf, L, r0, r1 - r0, full, spin)
            Hr, Sr = _oracle_rows(oracle, cf, L, spin, full, (r0, r1))
            assert H["index_ptr"][0] == 1 and S["index_ptr"][0] == 1
            assert h.block_count_rows(cf, L, r0, r1 - r0, full, spin) == (Hr["nnz"], Sr["nnz"])
            assert_csr_close(H, Hr, RTOL)
            assert_csr_close(S, Sr, RTOL, with_scale=False)


@pytest.mark.parametrize("stage_bytes", [64 << 10, 300 << 10])
def test_chunked_host_fill_matches_oracle(bs2e, oracle, stage_bytes):
    """Whole blocks through small staging areas (tens of chunks, the copy of
    one overlapping the fill of the next) equal the oracle."""
    for (L, spin) in [(1, 0), (3, 1)]:
        (L, M, par, spin, cf) = _case_block(bs2e, L, spin)
        Hr, Sr = _oracle_rows(oracle, cf, L, spin, True, None)
        assert 24 * (Hr["nnz"] + Sr["nnz"]) > 4 * stage_bytes  # several chunks
        with _handle(bs2e, stage_bytes=stage_bytes) as h:
            H, S = h.block(cf, L, True, spin)
            assert_csr_close(H, Hr, RTOL)
            assert_csr_close(S, Sr, RTOL, with_scale=False)
            # and a row range through the same small areas
            r0, r1 = cf.size // 5, cf.size // 2
            H2, S2 = h.block_rows(cf, L, r0, r1 - r0, True, spin)
            Hr2, Sr2 = _oracle_rows(oracle, cf, L, spin, True, (r0, r1))
            assert_csr_close(H2, Hr2, RTOL)
            assert_csr_close(S2, Sr2, RTOL, with_scale=False)


def test_mixed_chunked_rows(bs2e, oracle):
    (L, M, par, spin, cf) = _case_block(bs2e, 2, 0)
    r0, r1 = cf.size // 4, cf.size // 4 + 500
    Hr, Sr = _oracle_rows(oracle, cf, L, spin, True, (r0, r1))
    with _handle(bs2e, precision=bs2e.PREC_MIXED, stage_bytes=128 << 10) as h:
        H, S = h.block_rows(cf, L, r0, r1 - r0, True, spin)
    assert_csr_close(H, Hr, 1e-11)
    assert_csr_close(S, Sr, 1e-11, with_scale=False)


def test_device_row_range(bs2e, oracle):
    torch = pytest.importorskip("torch")
    (L, M, par, spin, cf) = _case_block(bs2e, 1, 1)
    r0, r1 = 40, cf.size - 35
    Hr, Sr = _oracle_rows(oracle, cf, L, spin, True, (r0, r1))
    dev = torch.device("cuda", 0)
    n = r1 - r0
    with _handle(bs2e) as h:
        nH, nS = h.block_count_rows(cf, L, r0, n, True, spin)
        Hd = dict(index_ptr=torch.empty(n + 1, dtype=torch.int64, device=dev),
                  indices=torch.empty(nH, dtype=torch.int64, device=dev),
                  data=torch.empty(nH, dtype=torch.complex128, device=dev))
        Sd = dict(index_ptr=torch.empty(n + 1, dtype=torch.int64, device=dev),
                  indices=torch.empty(nS, dtype=torch.int64, device=dev),
                  data=torch.empty(nS, dtype=torch.complex128, device=dev))
        h.block_rows_into(cf, L, r0, n, True, spin, {k: v.data_ptr() for k, v in Hd.items()},
                          {k: v.data_ptr() for k, v in Sd.items()})
        H = {k: v.cpu().numpy() for k, v in Hd.items()}
        S = {k: v.cpu().numpy() for k, v in Sd.items()}
    assert_csr_close(H, Hr, RTOL)
    assert_csr_close(S, Sr, RTOL, with_scale=False)


def test_row_range_errors(bs2e):
    (L, M, par, spin, cf) = _case_block(bs2e, 0, 0)
    with _handle(bs2e, stage_bytes=4096) as h:
        with pytest.raises(bs2e.Bs2eError, match="row range"):
            h.block_rows(cf, L, cf.size - 2, 5, True, spin)
        with pytest.raises(bs2e.Bs2eError, match="row range"):
            h.block_count_rows(cf, L, -1, 2, True, spin)
        with pytest.raises(bs2e.Bs2eError, match="staging area"):
            h.block(cf, L, True, spin)  # a row is larger than a 4 KiB area
        # the handle stays usable
        n_h, n_s = h.block_count_rows(cf, L, 0, 3, True, spin)
        assert n_h > 0


def test_row_mode_on_large_tiles(bs2e, oracle):
    """Order 9 with k=0..14 (35 KB R^k tiles): ranges inside one channel run a
    warp per row with the tile read through L1/L2; ranges across channels and
    whole blocks keep the staged tiles.  Both must give the oracle's rows."""
    c = CASES["bigtile"]
    ref = oracle_reference("bigtile")
    for prec, tol in ((0, RTOL), (bs2e.PREC_MIXED, 1e-11)):
        h = bs2e.Bs2e(ref["knots"], c["k"], c["q"], c["max_k"], precision=prec,
                      stage_bytes=96 << 10)
        try:
            h.slater()
            h.rk()
            h.set_one_body(ref["H1p"], ref["S"])
            for (L, M, par, spin, cf) in blocks(bs2e, "bigtile"):
                n = cf.size
                ch = cf["l1"] * 100 + cf["l2"]
                ends = np.flatnonzero(np.diff(ch)) + 1
                first_end = int(ends[0]) if ends.size else n  # end of the first channel
                for (r0, r1) in [(3, min(first_end, 60)), (0, n)]:
                    H, S = h.block_rows(cf, L, r0, r1 - r0, True, spin)
                    Hr, Sr = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"],
                                                    ref["H1p"], ref["S"], True, spin,
                                                    rows=(r0, r1))
                    assert_csr_close(H, Hr, tol)
                    assert_csr_close(S, Sr, tol, with_scale=False)
                # a whole block through 96 KiB staging areas (chunks inside channels)
                H, S = h.block(cf, L, True, spin)
                Hr, Sr = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"],
                                                ref["H1p"], ref["S"], True, spin)
                assert_csr_close(H, Hr, tol)
        finally:
            h.close()
