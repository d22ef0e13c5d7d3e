"""CPU tests of the oracle: pinned against golden vectors and analytic answers.

The reference's own tests assert nothing (tests/test_mat_els.f90 and
tests/test_gsl_3j.f90 only print), so the oracle is pinned here against exact
sympy 3j/6j values, numpy Gauss-Legendre nodes, hydrogenic Slater integrals
(the F0(1s,1s) = 5Z/8 ratio tests/test_mat_els.f90:179 prints) and the
symmetries of R^k.
"""
import json
import os

import numpy as np
import pytest
import scipy.linalg

from cases import CASES, blocks, knots, oracle_reference

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_gauss_legendre_vs_golden(oracle):
    gl = json.load(open(os.path.join(GOLD, "gauss_legendre.json")))
    for q, v in gl.items():
        x, w = oracle.gauss_legendre(int(q))
        np.testing.assert_allclose(x, v["x"], rtol=0, atol=4e-16)
        # the recurrence-based weight formula of the restated stdlib routine
        # carries ~1e-13 relative error at q ~ 20
        np.testing.assert_allclose(w, v["w"], rtol=2e-13, atol=0)


def test_gauss_legendre_exactness(oracle):
    # q-point rule integrates x^m exactly for m <= 2q-1
    for q in (3, 8, 10, 12):
        x, w = oracle.gauss_legendre(q)
        for m in range(2 * q):
            exact = 0.0 if m % 2 else 2.0 / (m + 1)
            assert abs(np.dot(w, x ** m) - exact) < 1e-14


def test_wigner_vs_golden(oracle):
    d = json.load(open(os.path.join(GOLD, "wigner.json")))
    for *a, v in d["three_j"]:
        assert abs(oracle.three_j(*a) - v) <= 1e-14 * max(1.0, abs(v)), a
    for *a, v in d["six_j"]:
        assert abs(oracle.six_j(*a) - v) <= 1e-13, a


def test_configs_match_reference_counts(oracle, bs2e):
    # rows of the order-6 N=60 l_max=2 singlet L=0 block, and the block sizes of
    # order 7, N=200, l_max=5, L=0..3
    assert oracle.count_configs(0, 0, 2, 60, 6).size == 5311
    for (L, par), n in {(0, 0): 117620, (1, 1): 195040, (2, 0): 253546, (3, 1): 272254}.items():
        assert oracle.count_configs(L, par, 5, 200, 7).size == n


def test_count_nnz_equals_construct(oracle, bs2e):
    for case in ("ref60", "small2", "cut"):
        c = CASES[case]
        ref = oracle_reference(case)
        for (L, M, par, spin, cf) in blocks(bs2e, case):
            for full in (True, False):
                nh, ns = oracle.count_nnz(cf, L, c["k"], c["max_k"], full, spin)
                H, S = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"],
                                              ref["H1p"], ref["S"], full, spin)
                assert (H["nnz"], S["nnz"]) == (nh, ns), (case, L, spin, full)
                assert H["index_ptr"][-1] == nh + 1


def _orbitals(oracle, t, k, q, Z, l):
    H = oracle.setup_H1p(t, k, q, Z, l + 1, cap_eta=0.0)[:, :, l].real
    S = oracle.setup_S(t, k, q).real
    e, v = scipy.linalg.eigh(H, S)
    return e, v  # columns S-normalised


def _slater(R, k, ca, cb, cc, cd, kk):
    """sum_abcd ca_a cb_b cc_c cd_d R^kk[a,b,c,d] (electron 1: a,c; electron 2: b,d)."""
    N = ca.size
    W = 2 * k - 1
    tot = 0.0
    for a in range(N):
        for b in range(N):
            for dc in range(W):
                c = a + dc - (k - 1)
                if c < 0 or c >= N:
                    continue
                row = R[a, b, dc, :, kk]
                d = b + np.arange(W) - (k - 1)
                ok = (d >= 0) & (d < N)
                tot += ca[a] * cb[b] * cc[c] * np.dot(row[ok], cd[d[ok]])
    return tot


def test_hydrogenic_slater_integrals(oracle):
    """F0(1s,1s)=5Z/8, F0(1s,2s)=17Z/81, G0(1s,2s)=16Z/729, F0(1s,2p)=59Z/243,
    G1(1s,2p)=112Z/2187 from the oracle's R^k store, He+ orbitals (Z=2) on the
    grid of the reference's tests/test_mat_els.f90:70-77 (k=8, m=3, h_max=1.5,
    r_max=15, k_GL=k+6).  The 2s/2p orbitals feel the r_max=15 wall at ~1e-9."""
    from conftest import load_package
    k, q, Z = 8, 14, 2
    t = load_package().grids.generate_grid(k, 3, Z, 1.5, 15.0)
    prim = oracle.slater(t, k, q, 1)
    R = oracle.rk_map(t.size - k - 2, k, 1, prim)
    e0, v0 = _orbitals(oracle, t, k, q, Z, 0)
    e1, v1 = _orbitals(oracle, t, k, q, Z, 1)
    assert abs(e0[0] + Z * Z / 2) < 1e-11 and abs(e0[1] + Z * Z / 8) < 1e-8
    assert abs(e1[0] + Z * Z / 8) < 1e-8
    s1, s2, p2 = v0[:, 0], v0[:, 1], v1[:, 0]
    checks = [((s1, s1, s1, s1, 0), 5 * Z / 8, 1e-11), ((s1, s2, s1, s2, 0), 17 * Z / 81, 1e-7),
              ((s1, s2, s2, s1, 0), 16 * Z / 729, 1e-7), ((s1, p2, s1, p2, 0), 59 * Z / 243, 1e-7),
              ((s1, p2, p2, s1, 1), 112 * Z / 2187, 1e-7)]
    for (a, b, c, d, kk), exact, tol in checks:
        val = _slater(R, k, a, b, c, d, kk)
        assert abs(abs(val) - exact) < tol * exact, (kk, val, exact)


def test_rk_symmetries_and_positivity(oracle, bs2e):
    c = CASES["ref60"]
    R = oracle_reference("ref60")["R"]
    k, N = c["k"], c["n_b"]
    rng = np.random.default_rng(3)
    keys = []
    while len(keys) < 3000:
        a, b = rng.integers(1, N + 1, 2)
        cc = a + rng.integers(-(k - 1), k)
        d = b + rng.integers(-(k - 1), k)
        if 1 <= cc <= N and 1 <= d <= N:
            keys.append((a, b, cc, d))
    keys = np.array(keys)
    v = oracle.rk_lookup(R, k, keys)
    assert (v > 0).all()
    for perm in ([2, 1, 0, 3], [0, 3, 2, 1], [1, 0, 3, 2]):
        w = oracle.rk_lookup(R, k, keys[:, perm])
        np.testing.assert_allclose(w, v, rtol=1e-13)


def test_block_symmetric_without_cap(oracle, bs2e):
    c = CASES["small2"]
    ref = oracle_reference("small2")
    for (L, M, par, spin, cf) in blocks(bs2e, "small2")[:3]:
        H, S = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"],
                                      ref["H1p"].real.astype(complex), ref["S"], True, spin)
        n = cf.size
        rows = np.repeat(np.arange(n), np.diff(H["index_ptr"]))
        cols = H["indices"] - 1
        A = {(i, j): v for i, j, v in zip(rows, cols, H["data"])}
        for (i, j), v in list(A.items())[::97]:
            assert abs(A[(j, i)] - v) <= 1e-12 * max(1.0, abs(v))


@pytest.mark.parametrize("case", ["ref60", "small2", "bigtile"])
def test_rk_tiles_equal_full_map(oracle, bs2e, case):
    """rk_tiles (whole R^k tiles straight from the knots, used where the full
    primitives are too slow) equals the full slater + rk_map store bit for
    bit on every tile, and the tile-table construct equals the banded one."""
    c = CASES[case]
    ref = oracle_reference(case)
    N, k = c["n_b"], c["k"]
    tiles = np.array([(a, b) for a in range(1, N + 1) for b in range(1, N + 1)])
    T = oracle.rk_tiles(ref["knots"], k, c["q"], c["max_k"], tiles)
    np.testing.assert_array_equal(T, ref["R"].reshape(N * N, *ref["R"].shape[2:]))
    for (L, M, par, spin, cf) in blocks(bs2e, case)[:2]:
        r0, r1 = 1, min(cf.size, 30)
        need = np.unique(np.stack([cf["n1"][r0:r1], cf["n2"][r0:r1]], 1), axis=0)
        Tn = oracle.rk_tiles(ref["knots"], k, c["q"], c["max_k"], need)
        args = (cf, L, k, N, c["max_k"])
        Ha, Sa = oracle.construct_block(*args, ref["R"], ref["H1p"], ref["S"], True, spin,
                                        rows=(r0, r1))
        Hb, Sb = oracle.construct_block(*args, Tn, ref["H1p"], ref["S"], True, spin,
                                        rows=(r0, r1), tile_of=oracle.tile_table(N, need))
        for x in ("index_ptr", "indices", "data", "scale"):
            np.testing.assert_array_equal(Ha[x], Hb[x])
        for x in ("index_ptr", "indices", "data"):
            np.testing.assert_array_equal(Sa[x], Sb[x])
    with pytest.raises(ValueError):
        oracle.construct_block(*args, Tn[:1], ref["H1p"], ref["S"], True, spin, rows=(r0, r1),
                               tile_of=oracle.tile_table(N, need[:1]))
