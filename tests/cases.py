"""Test cases shared by the CPU and GPU suites.

ref60 is the reference-sized CPU case (k=6, 60 B-splines on the exp-linear grid
to r_max=50, 8 GL points, k=0..4, singlet L=0 with l1=l2 in {0,1,2}).  small2
is the order-7 N=200 workload's method (k=7, 10 GL points, k=0..10, l_max=5, L=0..3, singlet and
triplet) on 30 B-splines so the O(n_config^2) oracle finishes in seconds.  cut
exercises the r_2_max / r_all_l / max_l2 cuts and the non-z-polarised
(unnatural parity) symmetry list.
"""
import functools

import numpy as np

CASES = {
    "ref60": dict(k=6, n_b=60, r_max=50.0, q=8, max_k=4, lmax=2, max_L=0, z_pol=True,
                 spins=(0,), Z=2),
    "small2": dict(k=7, n_b=30, r_max=30.0, q=10, max_k=10, lmax=5, max_L=3, z_pol=True,
                   spins=(0, 1), Z=2),
    "cut": dict(k=5, n_b=24, r_max=20.0, q=7, max_k=3, lmax=3, max_L=2, z_pol=False,
                spins=(0,), Z=2, max_n_b=15, n_all_l=12, l2_max=1),
    # radii to 1e5 a.u.: R^k slice maxima far below 2^-12, where the mixed
    # path joins the one-body and two-electron parts in FP64
    "wide": dict(k=6, n_b=28, r_max=1.0e5, q=8, max_k=6, lmax=2, max_L=1, z_pol=True,
                 spins=(0, 1), Z=2),
    # order 9 with k=0..14: 35 KB R^k tiles, where ranges inside one channel
    # run the fill a warp per row
    "bigtile": dict(k=9, n_b=24, r_max=30.0, q=9, max_k=14, lmax=2, max_L=1, z_pol=True,
                    spins=(0,), Z=2),
}


def knots(pkg, case):
    c = CASES[case]
    return pkg.grids.explin_knots(c["k"], c["n_b"], c["r_max"])


def blocks(pkg, case):
    """[(L, M, parity_odd, spin, configs)] of a case, configurations from the oracle."""
    import oracle as O
    c = CASES[case]
    out = []
    for spin in c["spins"]:
        for (L, M, par) in pkg.basis.symmetries(c["max_L"], c["z_pol"]):
            cf = O.count_configs(L, par, c["lmax"], c["n_b"], c["k"], c.get("max_n_b"),
                                 c.get("n_all_l"), c.get("l2_max"), spin)
            out.append((L, M, par, spin, cf))
    return out


@functools.lru_cache(maxsize=None)
def oracle_reference(case):
    """Oracle primitives, R^k map and one-body matrices of a case (cached)."""
    import oracle as O
    from conftest import load_package
    pkg = load_package()
    c = CASES[case]
    t = knots(pkg, case)
    prim = O.slater(t, c["k"], c["q"], c["max_k"])
    R = O.rk_map(c["n_b"], c["k"], c["max_k"], prim)
    H1p = O.setup_H1p(t, c["k"], c["q"], c["Z"], c["lmax"] + 1, cap_order=2, cap_r0=10.0,
                      cap_eta=1e-3)
    S = O.setup_S(t, c["k"], c["q"])
    return dict(knots=t, prim=prim, R=R, H1p=H1p, S=S)


def assert_csr_close(gpu, ref, rtol=1e-12, with_scale=True):
    """Bit-exact pattern, values within rtol of the oracle's term-magnitude scale."""
    np.testing.assert_array_equal(gpu["index_ptr"], ref["index_ptr"])
    np.testing.assert_array_equal(gpu["indices"], ref["indices"])
    g, r = gpu["data"], ref["data"]
    if with_scale and "scale" in ref:
        bound = rtol * ref["scale"]
    else:
        bound = rtol * np.maximum(np.abs(r), 1e-300)
    err = np.abs(g - r)
    bad = err > bound
    if bad.any():
        i = int(np.argmax(err - bound))
        raise AssertionError("%d of %d values off; worst at %d: gpu=%r ref=%r bound=%g" %
                             (bad.sum(), r.size, i, g[i], r[i], bound[i]))
