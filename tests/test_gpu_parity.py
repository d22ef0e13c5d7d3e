"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle.

Bars: CSR patterns and COO indices bit-exact; values within 1e-12 of the
oracle, relative to the magnitude of the entry's terms (a cancelling sum of
multipoles is compared against the size of its terms, not of its result).
"""
import numpy as np
import pytest

from cases import CASES, assert_csr_close, blocks, knots, oracle_reference

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _handle(bs2e, case, precision=0):
    c = CASES[case]
    h = bs2e.Bs2e(knots(bs2e, case), c["k"], c["q"], c["max_k"], precision=precision)
    h.slater()
    return h


@pytest.mark.parametrize("case", ["ref60", "small2", "cut"])
def test_primitives_match_oracle(bs2e, oracle, case):
    ref = oracle_reference(case)["prim"]
    with _handle(bs2e, case) as h:
        assert (h.nnz4, h.nnz6) == (ref["r_k"].shape[0], ref["r_d_k"].shape[0])
        g = h.primitives()
    np.testing.assert_array_equal(g["idx4"], ref["idx4"])
    np.testing.assert_array_equal(g["idx6"], ref["idx6"])
    for name in ("r_k", "r_m_k", "r_d_k"):
        np.testing.assert_allclose(g[name], ref[name], rtol=1e-13, atol=0, err_msg=name)


@pytest.mark.parametrize("case", ["ref60", "small2", "cut"])
def test_rk_store_matches_oracle(bs2e, oracle, case):
    c = CASES[case]
    R = oracle_reference(case)["R"]
    k, N, W = c["k"], c["n_b"], 2 * c["k"] - 1
    a, b, dc, dd = np.meshgrid(np.arange(N), np.arange(N), np.arange(W), np.arange(W),
                               indexing="ij")
    cc, d = a + dc - (k - 1), b + dd - (k - 1)
    ok = (cc >= 0) & (cc < N) & (d >= 0) & (d < N)
    keys = np.stack([a[ok] + 1, b[ok] + 1, cc[ok] + 1, d[ok] + 1], axis=1)
    with _handle(bs2e, case) as h:
        h.rk()
        got = h.rk_get(keys)
    want = oracle.rk_lookup(R, k, keys)
    assert (want > 0).all()
    np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)


def test_rk_partial_multipole_range(bs2e, oracle):
    c = CASES["small2"]
    R = oracle_reference("small2")["R"]
    keys = np.array([[3, 9, 5, 12], [10, 10, 14, 7], [1, 30, 6, 25], [15, 16, 15, 16]])
    with _handle(bs2e, "small2") as h:
        for k0 in range(0, c["max_k"] + 1, 4):
            h.rk(k0, min(4, c["max_k"] + 1 - k0))
        got = h.rk_get(keys)
    np.testing.assert_allclose(got, oracle.rk_lookup(R, c["k"], keys), rtol=RTOL)


@pytest.mark.parametrize("case", ["ref60", "small2"])
def test_one_body_matches_oracle(bs2e, oracle, case):
    c = CASES[case]
    ref = oracle_reference(case)
    with _handle(bs2e, case) as h:
        H, S = h.one_body(c["Z"], c["lmax"] + 1, 2, 10.0, 1e-3)
    np.testing.assert_allclose(S, ref["S"], rtol=0, atol=1e-14 * np.abs(ref["S"]).max())
    for l in range(c["lmax"] + 1):
        scale = np.abs(ref["H1p"][:, :, l]).max()
        np.testing.assert_allclose(H[:, :, l], ref["H1p"][:, :, l], rtol=0, atol=1e-12 * scale)


@pytest.mark.parametrize("case", ["ref60", "small2", "cut"])
@pytest.mark.parametrize("full", [True, False])
def test_blocks_match_oracle(bs2e, oracle, case, full):
    c = CASES[case]
    ref = oracle_reference(case)
    with _handle(bs2e, case) as h:
        h.rk()
        h.set_one_body(ref["H1p"], ref["S"])
        for (L, M, par, spin, cf) in blocks(bs2e, case):
            nh, ns = h.block_count(cf, L, full, spin)
            assert (nh, ns) == oracle.count_nnz(cf, L, c["k"], c["max_k"], full, spin)
            Hg, Sg = h.block(cf, L, full, spin)
            Hr, Sr = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"],
                                            ref["H1p"], ref["S"], full, spin)
            assert_csr_close(Hg, Hr, RTOL)
            assert_csr_close(Sg, Sr, RTOL, with_scale=False)


@pytest.mark.parametrize("case", ["small2", "cut"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_blocks_with_complex_overlap_match_oracle(bs2e, oracle, case, prec):
    """A complex overlap matrix (as a complex-scaled radial grid gives) takes the
    fill's complex-S branches of S_mat_neq and H_1p_neq (mat_els.f90:664-715)."""
    c = CASES[case]
    ref = oracle_reference(case)
    S = ref["S"] * (1.0 + 0.3j)
    precision = bs2e.PREC_FP64 if prec == "fp64" else bs2e.PREC_MIXED
    tol = RTOL if prec == "fp64" else 1e-11
    with _handle(bs2e, case, precision=precision) as h:
        h.rk()
        h.set_one_body(ref["H1p"], S)
        for (L, M, par, spin, cf) in blocks(bs2e, case):
            for full in (True, False):
                Hg, Sg = h.block(cf, L, full, spin)
                Hr, Sr = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"],
                                                ref["H1p"], S, full, spin)
                assert_csr_close(Hg, Hr, tol)
                assert_csr_close(Sg, Sr, tol, with_scale=False)


def test_device_outputs_match_host_outputs(bs2e, oracle):
    import torch
    c = CASES["small2"]
    ref = oracle_reference("small2")
    (L, M, par, spin, cf) = blocks(bs2e, "small2")[2]
    with _handle(bs2e, "small2") as h:
        h.rk()
        h.set_one_body(ref["H1p"], ref["S"])
        Hh, Sh = h.block(cf, L, True, spin)
        n = cf.size
        dev = torch.device("cuda:0")
        Ht = dict(index_ptr=torch.zeros(n + 1, dtype=torch.int64, device=dev),
                  indices=torch.zeros(Hh["nnz"], dtype=torch.int64, device=dev),
                  data=torch.zeros(Hh["nnz"], dtype=torch.complex128, device=dev))
        St = dict(index_ptr=torch.zeros(n + 1, dtype=torch.int64, device=dev),
                  indices=torch.zeros(Sh["nnz"], dtype=torch.int64, device=dev),
                  data=torch.zeros(Sh["nnz"], dtype=torch.complex128, device=dev))
        torch.cuda.synchronize()
        h.block_fill_into(cf, L, True, spin, {x: t.data_ptr() for x, t in Ht.items()},
                          {x: t.data_ptr() for x, t in St.items()}, on_device=True)
    for x in ("index_ptr", "indices", "data"):
        np.testing.assert_array_equal(Ht[x].cpu().numpy(), Hh[x])
        np.testing.assert_array_equal(St[x].cpu().numpy(), Sh[x])


def test_empty_block_and_error_paths(bs2e, oracle):
    c = CASES["ref60"]
    ref = oracle_reference("ref60")
    with _handle(bs2e, "ref60") as h:
        cf = np.zeros(0, dtype=bs2e.CONFIG_DTYPE)
        with pytest.raises(bs2e.Bs2eError) as e:  # R^k not built yet
            h.block(cf, 0)
        assert e.value.status == 6
        h.rk()
        h.set_one_body(ref["H1p"], ref["S"])
        H, S = h.block(cf, 0)
        assert H["nnz"] == 0 and list(H["index_ptr"]) == [1]
        good = blocks(bs2e, "ref60")[0][4]
        bad = np.concatenate([good[good["l1"] == 1], good[good["l1"] == 0]])
        bad = np.concatenate([bad, good[good["l1"] == 1][:1]])  # channel (1,1) split in two
        with pytest.raises(bs2e.Bs2eError) as e:
            h.block(bad, 0)
        assert e.value.status == 8
        # the handle stays usable after an error
        H2, _ = h.block(good, 0)
        assert H2["nnz"] == oracle.count_nnz(good, 0, c["k"], c["max_k"])[0]


def test_gpu_hydrogenic_known_answer(bs2e, oracle):
    """F0(1s,1s) = 5Z/8 from the GPU R^k store (reference test grid, k=8)."""
    import scipy.linalg
    k, q, Z = 8, 14, 2
    t = bs2e.grids.generate_grid(k, 3, Z, 1.5, 15.0)
    with bs2e.Bs2e(t, k, q, 0) as h:
        h.slater()
        h.rk()
        H, S = h.one_body(Z, 1, 2, 1e9, 0.0)
        N = h.n_b
        e, v = scipy.linalg.eigh(H[:, :, 0].real, S.real)
        c1 = v[:, 0]
        W = 2 * k - 1
        a, b, dc, dd = np.meshgrid(np.arange(N), np.arange(N), np.arange(W), np.arange(W),
                                   indexing="ij")
        cc, d = a + dc - (k - 1), b + dd - (k - 1)
        ok = (cc >= 0) & (cc < N) & (d >= 0) & (d < N)
        keys = np.stack([a[ok], b[ok], cc[ok], d[ok]], axis=1)
        vals = h.rk_get(keys + 1)[:, 0]
    F0 = np.sum(c1[keys[:, 0]] * c1[keys[:, 1]] * c1[keys[:, 2]] * c1[keys[:, 3]] * vals)
    assert abs(e[0] + Z * Z / 2) < 1e-11
    assert abs(F0 - 5 * Z / 8) < 1e-11 * (5 * Z / 8)


# ---------------------------------------------------------------------------
# Mixed path: R^k stored as scaled FP32 pairs, multipole sums in FP32-pair
# arithmetic.  Target <= 1e-9 relative (term-magnitude scale); the pairs carry
# ~44 bits, so the bar checked here is 1e-11.
# ---------------------------------------------------------------------------
MIXED_RTOL = 1e-11


@pytest.mark.parametrize("case", ["ref60", "small2", "wide"])
def test_mixed_rk_store_matches_oracle(bs2e, oracle, case):
    c = CASES[case]
    R = oracle_reference(case)["R"]
    k, N, W = c["k"], c["n_b"], 2 * c["k"] - 1
    a, b, dc, dd = np.meshgrid(np.arange(N), np.arange(N), np.arange(W), np.arange(W),
                               indexing="ij")
    cc, d = a + dc - (k - 1), b + dd - (k - 1)
    ok = (cc >= 0) & (cc < N) & (d >= 0) & (d < N)
    keys = np.stack([a[ok] + 1, b[ok] + 1, cc[ok] + 1, d[ok] + 1], axis=1)
    with _handle(bs2e, case, precision=bs2e.PREC_MIXED) as h:
        h.rk()
        got = h.rk_get(keys)
    np.testing.assert_allclose(got, oracle.rk_lookup(R, k, keys), rtol=1e-13, atol=0)


@pytest.mark.parametrize("case", ["ref60", "small2", "cut", "wide"])
def test_mixed_blocks_match_oracle(bs2e, oracle, case):
    c = CASES[case]
    ref = oracle_reference(case)
    worst = 0.0
    with _handle(bs2e, case, precision=bs2e.PREC_MIXED) as h:
        h.rk()
        h.set_one_body(ref["H1p"], ref["S"])
        for (L, M, par, spin, cf) in blocks(bs2e, case):
            Hg, Sg = h.block(cf, L, True, spin)
            Hr, Sr = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"],
                                            ref["H1p"], ref["S"], True, spin)
            assert_csr_close(Hg, Hr, MIXED_RTOL)
            assert_csr_close(Sg, Sr, RTOL, with_scale=False)
            rel = np.abs(Hg["data"] - Hr["data"]) / np.maximum(Hr["scale"], 1e-300)
            worst = max(worst, float(rel.max()) if rel.size else 0.0)
    print("mixed %s: max error / term scale = %.3e" % (case, worst))


# ---------------------------------------------------------------------------
# Dipole blocks (construct_dip_block_tensor, src/mat_els/dipole.f90:8-146)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("gauge", [0, 1])
def test_radial_dipole_matches_oracle(bs2e, oracle, gauge):
    c = CASES["small2"]
    t = knots(bs2e, "small2")
    want = oracle.setup_radial_dip(t, c["k"], c["q"], gauge)
    with _handle(bs2e, "small2") as h:
        got = h.radial_dipole(gauge)
    for g, w in zip(got, want):
        np.testing.assert_allclose(g, w, rtol=0, atol=1e-13 * np.abs(w).max())


@pytest.mark.parametrize("case", ["small2", "cut"])
@pytest.mark.parametrize("gauge", [0, 1])
def test_dipole_blocks_match_oracle(bs2e, oracle, case, gauge):
    c = CASES[case]
    ref = oracle_reference(case)
    mats = oracle.setup_radial_dip(ref["knots"], c["k"], c["q"], gauge)
    bl = [b for b in blocks(bs2e, case) if b[3] == 0]
    n_checked = 0
    with _handle(bs2e, case) as h:
        h.set_one_body(ref["H1p"], ref["S"])
        if gauge == 0:
            h.set_radial_dipole(0, r_mat=mats[0])
        else:
            h.set_radial_dipole(1, dr_mat=mats[0], r_inv_mat=mats[1])
        for q in (-1, 0, 1):
            for j, (L2, M2, p2, _, cols) in enumerate(bl):
                for i, (L1, M1, p1, _, rows) in enumerate(bl):
                    compute = not (i > j and case == "cut")  # full=.false. skips i > j
                    want = oracle.dip_block(rows, (L1, M1, p1), cols, (L2, M2, p2), q, compute,
                                            c["k"], c["n_b"], gauge, ref["S"], mats)
                    got = h.dip_block(rows, (L1, M1, p1), cols, (L2, M2, p2), q, compute)
                    assert got["nnz"] == want["nnz"]
                    np.testing.assert_array_equal(got["index_ptr"], want["index_ptr"])
                    np.testing.assert_array_equal(got["indices"], want["indices"])
                    scale = max(np.abs(want["data"]).max() if want["nnz"] else 0.0, 1e-300)
                    np.testing.assert_allclose(got["data"], want["data"], rtol=0,
                                               atol=1e-12 * scale)
                    n_checked += want["nnz"] > 0
    assert n_checked > 0


def test_device_radial_dipole_drives_blocks(bs2e, oracle):
    c = CASES["small2"]
    ref = oracle_reference("small2")
    mats = oracle.setup_radial_dip(ref["knots"], c["k"], c["q"], 1)
    bl = [b for b in blocks(bs2e, "small2") if b[3] == 0]
    (L1, M1, p1, _, rows), (L2, M2, p2, _, cols) = bl[0], bl[1]
    with _handle(bs2e, "small2") as h:
        h.set_one_body(ref["H1p"], ref["S"])
        h.radial_dipole(1, copy_out=False)
        got = h.dip_block(rows, (L1, M1, p1), cols, (L2, M2, p2), 0)
    want = oracle.dip_block(rows, (L1, M1, p1), cols, (L2, M2, p2), 0, True, c["k"], c["n_b"], 1,
                            ref["S"], mats)
    np.testing.assert_array_equal(got["indices"], want["indices"])
    np.testing.assert_allclose(got["data"], want["data"], rtol=0,
                               atol=1e-12 * np.abs(want["data"]).max())


def test_dipole_blocks_with_complex_bands_match_oracle(bs2e, oracle):
    """Radial dipole bands with both real and imaginary parts (a caller's own
    matrices) take the fill's general complex arithmetic; the library's own
    bands are real (length gauge) or imaginary (velocity gauge) and take the
    real-arithmetic forms checked above."""
    c = CASES["small2"]
    ref = oracle_reference("small2")
    mats = oracle.setup_radial_dip(ref["knots"], c["k"], c["q"], 0)
    r_mat = np.asarray(mats[0]) * (0.8 + 0.6j)
    mats_c = (r_mat,) + tuple(mats[1:])
    bl = [b for b in blocks(bs2e, "small2") if b[3] == 0]
    (L1, M1, p1, _, rows), (L2, M2, p2, _, cols) = bl[0], bl[1]
    with _handle(bs2e, "small2") as h:
        h.set_one_body(ref["H1p"], ref["S"])
        h.set_radial_dipole(0, r_mat=r_mat)
        n_checked = 0
        for q in (-1, 0, 1):
            want = oracle.dip_block(rows, (L1, M1, p1), cols, (L2, M2, p2), q, True, c["k"],
                                    c["n_b"], 0, ref["S"], mats_c)
            got = h.dip_block(rows, (L1, M1, p1), cols, (L2, M2, p2), q, True)
            assert got["nnz"] == want["nnz"]
            if want["nnz"] == 0:
                continue
            n_checked += 1
            np.testing.assert_array_equal(got["indices"], want["indices"])
            scale = np.abs(want["data"]).max()
            np.testing.assert_allclose(got["data"], want["data"], rtol=0, atol=1e-12 * scale)
            assert np.abs(got["data"].imag).max() > 0.1 * scale  # the imaginary parts are there
        assert n_checked > 0
