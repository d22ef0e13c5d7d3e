"""n1 bands of a block (bs2e_block_band_count / bs2e_block_fill_band) and the
block-cache setting (bs2e_set_block_cache), through the C ABI.

A band holds the rows of every channel with n1 in a range, in block order; its
CSR must equal those rows of the whole block bit for bit (same kernel, other
output positions), its counts must add up to the block's, and it must match
the oracle on the same rows.  With the block cache off, cycling through the
blocks re-plans and recounts each (the count kernel runs again) and gives the
same counts.
"""
import numpy as np
import pytest

from cases import CASES, blocks, knots, oracle_reference, assert_csr_close

pytestmark = pytest.mark.gpu


def _dev_band(torch, h, cf, L, spin, a, m):
    dev = torch.device("cuda", 0)
    r, nh, ns = h.band_count(cf, L, a, m, True, spin)
    mk = lambda n, dt: torch.empty(max(int(n), 1), dtype=dt, device=dev)
    H = dict(index_ptr=mk(r + 1, torch.int64), indices=mk(nh, torch.int64),
             data=mk(nh, torch.complex128))
    S = dict(index_ptr=mk(r + 1, torch.int64), indices=mk(ns, torch.int64),
             data=mk(ns, torch.complex128))
    rows = mk(r, torch.int64)
    torch.cuda.synchronize()
    h.band_into(cf, L, a, m, True, spin, {x: v.data_ptr() for x, v in H.items()},
                {x: v.data_ptr() for x, v in S.items()}, rows.data_ptr())
    out = lambda d, n: {"index_ptr": d["index_ptr"][:r + 1].cpu().numpy(),
                        "indices": d["indices"][:n].cpu().numpy(),
                        "data": d["data"][:n].cpu().numpy()}
    return out(H, nh), out(S, ns), rows[:r].cpu().numpy(), (r, nh, ns)


def _rows_of(M, rows0):
    """CSR of the given 0-based rows of a whole-block CSR (1-based arrays)."""
    ptr, idx, dat = M["index_ptr"], M["indices"], M["data"]
    lens = ptr[rows0 + 1] - ptr[rows0]
    sel = np.concatenate([np.arange(ptr[r] - 1, ptr[r + 1] - 1) for r in rows0]) if len(rows0) \
        else np.zeros(0, np.int64)
    return {"index_ptr": np.concatenate([[1], 1 + np.cumsum(lens)]), "indices": idx[sel],
            "data": dat[sel]}


@pytest.mark.parametrize("precision", [0, 1])
def test_bands_equal_block_rows(bs2e, oracle, precision):
    torch = pytest.importorskip("torch")
    c = CASES["small2"]
    ref = oracle_reference("small2")
    N = c["n_b"]
    with bs2e.Bs2e(knots(bs2e, "small2"), c["k"], c["q"], c["max_k"], precision=precision) as h:
        h.slater()
        h.rk()
        h.set_one_body(ref["H1p"], ref["S"])
        for (L, M, par, spin, cf) in blocks(bs2e, "small2"):
            Hb, Sb = h.block(cf, L, True, spin)
            r_all, h_all, s_all, per = h.band_count(cf, L, 1, N, True, spin, per_n1=True)
            assert (r_all, h_all, s_all) == (cf.size, Hb["nnz"], Sb["nnz"])
            assert per[:, 0].sum() == cf.size and per[:, 1].sum() == Hb["nnz"]
            for n1 in (1, 7, N):  # per-n1 counts equal the rows with that n1
                assert per[n1 - 1, 0] == int((cf["n1"] == n1).sum())
            for (a, m) in ((1, N), (1, 4), (5, 9), (14, 1), (N, 1), (N - 2, 10), (N + 3, 2),
                           (-3, 5), (3, 0)):
                H, S, rows, (r, nh, ns) = _dev_band(torch, h, cf, L, spin, a, m)
                want = np.flatnonzero((cf["n1"] >= a) & (cf["n1"] < a + m))
                np.testing.assert_array_equal(rows, want + 1)
                for got, full in ((H, Hb), (S, Sb)):
                    w = _rows_of(full, want)
                    for x in ("index_ptr", "indices", "data"):
                        np.testing.assert_array_equal(got[x], w[x])
                if (a, m) == (5, 9):  # the same band into host arrays
                    rows_h, Hh, Sh = h.band(cf, L, a, m, True, spin)
                    np.testing.assert_array_equal(rows_h, rows)
                    for got, dv in ((Hh, H), (Sh, S)):
                        for x in ("index_ptr", "indices", "data"):
                            np.testing.assert_array_equal(got[x], dv[x])
            # the whole block (which the bands reproduce) against the oracle
            Hr, Sr = oracle.construct_block(cf, L, c["k"], N, c["max_k"], ref["R"], ref["H1p"],
                                            ref["S"], True, spin)
            assert_csr_close(Hb, Hr, rtol=1e-12 if precision == 0 else 1e-11)


def test_block_cache_off_recounts(bs2e):
    c = CASES["small2"]
    with bs2e.Bs2e(knots(bs2e, "small2"), c["k"], c["q"], c["max_k"]) as h:
        h.slater()
        h.rk()
        bl = blocks(bs2e, "small2")
        first = [h.block_count(cf, L, True, spin) for (L, M, par, spin, cf) in bl]
        n0 = h.launch_count
        again = [h.block_count(cf, L, True, spin) for (L, M, par, spin, cf) in bl]
        cached = h.launch_count - n0  # cache hits: compare kernels only
        h.set_block_cache(0)
        n0 = h.launch_count
        off = [h.block_count(cf, L, True, spin) for (L, M, par, spin, cf) in bl]
        recount = h.launch_count - n0
        assert first == again == off
        # kept blocks cost one compare kernel each; without the cache every
        # block runs its channel-marks, segment-plan and count kernels again
        assert cached == len(bl)
        assert recount >= 3 * len(bl)
        with pytest.raises(bs2e.Bs2eError):
            h.set_block_cache(17)
        h.set_block_cache(16)
        assert [h.block_count(cf, L, True, spin) for (L, M, par, spin, cf) in bl] == first


def test_host_band_larger_than_staging_is_refused(bs2e):
    """A band whose slice of one channel exceeds a staging area is refused
    with a message that names the staging area; narrower bands still fill."""
    c = CASES["small2"]
    with bs2e.Bs2e(knots(bs2e, "small2"), c["k"], c["q"], c["max_k"], stage_bytes=65536) as h:
        h.slater()
        h.rk()
        h.one_body(c["Z"], c["lmax"] + 1)
        L, M, par, spin, cf = blocks(bs2e, "small2")[0]
        with pytest.raises(bs2e.Bs2eError) as e:
            h.band(cf, L, 1, c["n_b"], True, spin)
        assert e.value.status == 1 and "staging" in str(e.value)
        rows, H, S = h.band(cf, L, 1, 1, True, spin)  # one n1 of the first channel fits
        assert rows.size == int((cf["n1"] == 1).sum())


def test_host_band_in_channel_groups_equals_device_band(bs2e):
    """A band larger than one staging area, filled into host arrays in groups
    of whole channels through the two staging areas (fill of one group beside
    the copy of the previous), equals the device-output band bit for bit."""
    torch = pytest.importorskip("torch")
    c = CASES["small2"]
    ref = oracle_reference("small2")
    bl = blocks(bs2e, "small2")
    L, M, par, spin, cf = max(bl, key=lambda b: b[4].size)
    with bs2e.Bs2e(knots(bs2e, "small2"), c["k"], c["q"], c["max_k"]) as hd:
        hd.slater()
        hd.rk()
        hd.set_one_body(ref["H1p"], ref["S"])
        Hd, Sd, rows_d, (r, nh, ns) = _dev_band(torch, hd, cf, L, spin, 1, c["n_b"])
    total = 40 * (nh + ns)
    done = False
    for div in (6, 4, 3, 2):
        stage = max(total // div, 4096)
        with bs2e.Bs2e(knots(bs2e, "small2"), c["k"], c["q"], c["max_k"],
                       stage_bytes=stage) as h:
            h.slater()
            h.rk()
            h.set_one_body(ref["H1p"], ref["S"])
            try:
                rows, H, S = h.band(cf, L, 1, c["n_b"], True, spin)
            except bs2e.Bs2eError as e:
                assert "staging" in str(e)
                continue
        assert stage < 24 * (nh + ns)  # so the band took several groups
        for A, B in ((H, Hd), (S, Sd)):
            for key in ("index_ptr", "indices"):
                np.testing.assert_array_equal(A[key], B[key])
            np.testing.assert_array_equal(A["data"].view(np.int64), B["data"].view(np.int64))
        np.testing.assert_array_equal(rows, rows_d)
        done = True
        break
    assert done, "no staging size between a sixth and half of the band worked"
