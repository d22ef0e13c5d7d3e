"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: the oracle is the FP64 CPU restatement of the
reference Fortran used to check the GPU library and as the timed CPU baseline.
Only tests/, the smoke check and the CPU-baseline leg of bench.py use it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

CONFIG_DTYPE = np.dtype([("n1", "<i8"), ("n2", "<i8"), ("l1", "<i8"), ("l2", "<i8"),
                         ("eqv", "<i8")])

_lib = None


def build():
    r = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = ctypes.CDLL(LIB_PATH)
    i64, p, dbl = ctypes.c_int64, ctypes.c_void_p, ctypes.c_double
    sig = {
        "or_gauss_legendre": (None, [i64, p, p]),
        "or_bvalue": (dbl, [p, i64, i64, dbl, i64, i64, i64]),
        "or_three_j": (dbl, [i64] * 6),
        "or_six_j": (dbl, [i64] * 6),
        "or_C_red_mat": (dbl, [i64] * 3),
        "or_ang_k_LS": (dbl, [i64] * 6),
        "or_nnz4": (i64, [i64, i64]),
        "or_nnz6": (i64, [i64, i64]),
        "or_slater": (None, [p, i64, i64, i64, i64, p, p, p, p, p, ctypes.c_int]),
        "or_rk_map": (None, [i64, i64, i64, i64, p, p, p, i64, p, p, p]),
        "or_count_configs": (i64, [i64] * 9 + [p]),
        "or_count_nnz": (None, [p, i64, i64, i64, i64, i64, i64, p]),
        "or_construct_block": (None, [p, i64, i64, i64, i64, i64, i64, i64, p, p, i64, p, i64,
                                      i64, p, p, p, p, p, p, p, p]),
        "or_construct_block_tiles": (None, [p, i64, i64, i64, i64, i64, i64, i64, p, p, p, i64,
                                            p, i64, i64, p, p, p, p, p, p, p, p]),
        "or_rk_tiles": (None, [p, i64, i64, i64, i64, i64, p, p, ctypes.c_int]),
        "or_setup_S": (None, [p, i64, i64, i64, p]),
        "or_setup_H1p": (None, [p, i64, i64, i64, i64, i64, i64, dbl, dbl, dbl, p]),
        "or_setup_radial_dip": (None, [p, i64, i64, i64, i64, p, p, p]),
        "or_dip_block": (i64, [p, i64, i64, i64, i64, p, i64, i64, i64, i64, i64, i64, i64, i64,
                               i64, p, p, p, p, p, p, p]),
        "or_csr_mv": (None, [i64, i64, i64, p, p, p, p, p, p]),
        "or_csr_from_blocks": (i64, [i64, i64, p, p, p, p, p, p, p, p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def gauss_legendre(q):
    x, w = np.zeros(q), np.zeros(q)
    lib().or_gauss_legendre(q, _p(x), _p(w))
    return x, w


def bvalue(knots, k, x, iv, jspline, ideriv=0):
    t = np.ascontiguousarray(knots, dtype=np.float64)
    return lib().or_bvalue(_p(t), t.size - k, k, float(x), ideriv, iv, jspline)


def three_j(*a):
    return lib().or_three_j(*a)


def six_j(*a):
    return lib().or_six_j(*a)


def ang_k_LS(k, la, lb, lc, ld, L):
    return lib().or_ang_k_LS(k, la, lb, lc, ld, L)


def slater(knots, k, k_GL, max_k, nthreads=0):
    """setup_Slater_integrals: COO arrays in the reference's order."""
    t = np.ascontiguousarray(knots, dtype=np.float64)
    L = lib()
    n4, n6 = L.or_nnz4(t.size, k), L.or_nnz6(t.size, k)
    K1 = max_k + 1
    rk = np.zeros((n4, K1), order="F")
    rmk = np.zeros((n4, K1), order="F")
    i4 = np.zeros((n4, 3), dtype=np.int64)
    rdk = np.zeros((n6, K1), order="F")
    i6 = np.zeros((n6, 5), dtype=np.int64)
    L.or_slater(_p(t), t.size, k, k_GL, max_k, _p(rk), _p(rmk), _p(i4), _p(rdk), _p(i6),
                int(nthreads))
    return dict(r_k=rk, r_m_k=rmk, idx4=i4, r_d_k=rdk, idx6=i6)


def rk_map(n_b, k, max_k, prim):
    """compute_R_k_map; banded array R[a][b][c-a+k-1][d-b+k-1][kk] (0-based a, b)."""
    W = 2 * k - 1
    R = np.zeros((n_b, n_b, W, W, max_k + 1))
    p = prim
    lib().or_rk_map(n_b, k, max_k, p["idx4"].shape[0], _p(p["r_k"]), _p(p["r_m_k"]),
                    _p(p["idx4"]), p["idx6"].shape[0], _p(p["r_d_k"]), _p(p["idx6"]), _p(R))
    return R


def rk_lookup(R, k, keys):
    """Values of 1-based keys [a,b,c,d] from a banded oracle store."""
    keys = np.asarray(keys, dtype=np.int64).reshape(-1, 4)
    a, b, c, d = (keys[:, i] - 1 for i in range(4))
    return R[a, b, c - a + k - 1, d - b + k - 1, :]


def count_configs(L, parity_odd, max_l_1p, n_b, k, max_n_b=None, n_all_l=None, l2_max=None,
                  spin=0):
    max_n_b = n_b if max_n_b is None else max_n_b
    n_all_l = n_b if n_all_l is None else n_all_l
    l2_max = max_l_1p if l2_max is None else l2_max
    args = [L, int(parity_odd), max_l_1p, n_b, k, max_n_b, n_all_l, l2_max, spin]
    n = lib().or_count_configs(*args, None)
    out = np.zeros(n, dtype=CONFIG_DTYPE)
    lib().or_count_configs(*args, _p(out))
    return out


def count_nnz(cf, L, k, max_k, full=True, spin=0):
    cf = np.ascontiguousarray(cf)
    nnz = np.zeros(2, dtype=np.int64)
    lib().or_count_nnz(_p(cf), cf.size, L, spin, k, max_k, int(bool(full)), _p(nnz))
    return int(nnz[0]), int(nnz[1])


def rk_tiles(knots, k, k_GL, max_k, tiles, nthreads=0):
    """R^k of whole tiles (a, b) (1-based pairs, n x 2) straight from the
    knots: array (n, W, W, max_k+1) laid out like rk_map's R[a-1, b-1], each
    value equal to rk_map's bit for bit (same primitives, same summation
    order), without the full O(N^2 k^4) primitives."""
    t = np.ascontiguousarray(knots, dtype=np.float64)
    ab = np.ascontiguousarray(np.asarray(tiles, dtype=np.int64).reshape(-1, 2))
    W = 2 * k - 1
    out = np.zeros((ab.shape[0], W, W, max_k + 1))
    lib().or_rk_tiles(_p(t), t.size, k, k_GL, max_k, ab.shape[0], _p(ab), _p(out), int(nthreads))
    return out


def tile_table(n_b, tiles):
    """tile_of[(a-1)*n_b + (b-1)] = index of tile (a, b) in a rk_tiles array, -1 elsewhere."""
    ab = np.asarray(tiles, dtype=np.int64).reshape(-1, 2)
    tab = np.full(n_b * n_b, -1, dtype=np.int64)
    tab[(ab[:, 0] - 1) * n_b + (ab[:, 1] - 1)] = np.arange(ab.shape[0])
    return tab


def construct_block(cf, L, k, n_b, max_k, R, H1p, S, full=True, spin=0, rows=None,
                    tile_of=None):
    """construct_block_tensor for rows [r0, r1) (default: all).  Returns (H, S)
    dicts with 1-based CSR arrays local to the row range; H['scale'] holds the
    sum of magnitudes of the terms of each entry.  R is the banded rk_map
    store, or (with tile_of from tile_table) a rk_tiles array holding the tile
    (n1, n2) of every row of the range."""
    cf = np.ascontiguousarray(cf)
    r0, r1 = (0, cf.size) if rows is None else rows
    R = np.ascontiguousarray(R, dtype=np.float64)
    H1p = np.asfortranarray(H1p, dtype=np.complex128)
    S = np.asfortranarray(S, dtype=np.complex128)
    n_l = H1p.shape[2] if H1p.ndim == 3 else 1
    L_ = lib()
    nnz = np.zeros(2, dtype=np.int64)
    if tile_of is not None:
        tile_of = np.ascontiguousarray(tile_of, dtype=np.int64)
        args = [_p(cf), cf.size, L, spin, k, n_b, max_k, int(bool(full)), _p(R), _p(tile_of),
                _p(H1p), n_l, _p(S), r0, r1]
        fn = L_.or_construct_block_tiles
    else:
        args = [_p(cf), cf.size, L, spin, k, n_b, max_k, int(bool(full)), _p(R), _p(H1p), n_l,
                _p(S), r0, r1]
        fn = L_.or_construct_block
    fn(*args, None, None, None, None, None, None, None, _p(nnz))
    if nnz[0] < 0:
        raise ValueError("construct_block: a row's R^k tile is not in the tile table")
    nh, ns = int(nnz[0]), int(nnz[1])
    n = r1 - r0
    H = dict(index_ptr=np.zeros(n + 1, np.int64), indices=np.zeros(nh, np.int64),
             data=np.zeros(nh, np.complex128), scale=np.zeros(nh), nnz=nh)
    Sd = dict(index_ptr=np.zeros(n + 1, np.int64), indices=np.zeros(ns, np.int64),
              data=np.zeros(ns, np.complex128), nnz=ns)
    fn(*args, _p(H["index_ptr"]), _p(H["indices"]), _p(H["data"]),
                          _p(H["scale"]), _p(Sd["index_ptr"]), _p(Sd["indices"]),
                          _p(Sd["data"]), _p(nnz))
    return H, Sd


def setup_S(knots, k, k_GL):
    t = np.ascontiguousarray(knots, dtype=np.float64)
    nb = t.size - k - 2
    S = np.zeros((nb, nb), dtype=np.complex128, order="F")
    lib().or_setup_S(_p(t), t.size, k, k_GL, _p(S))
    return S


def setup_H1p(knots, k, k_GL, Z, n_l, cap_order=2, cap_r0=10.0, cap_eta=1e-3 + 0j):
    t = np.ascontiguousarray(knots, dtype=np.float64)
    nb = t.size - k - 2
    H = np.zeros((nb, nb, n_l), dtype=np.complex128, order="F")
    eta = complex(cap_eta)
    for l in range(n_l):
        Hl = np.zeros((nb, nb), dtype=np.complex128, order="F")
        lib().or_setup_H1p(_p(t), t.size, k, k_GL, Z, l, cap_order, float(cap_r0), eta.real,
                           eta.imag, _p(Hl))
        H[:, :, l] = Hl
    return H


def setup_radial_dip(knots, k, k_GL, gauge):
    """(r_mat,) for the length gauge, (dr_mat, r_inv_mat) for the velocity gauge."""
    t = np.ascontiguousarray(knots, dtype=np.float64)
    nb = t.size - k - 2
    mk = lambda: np.zeros((nb, nb), dtype=np.complex128, order="F")
    r, d, ri = mk(), mk(), mk()
    lib().or_setup_radial_dip(_p(t), t.size, k, k_GL, int(gauge), _p(r), _p(d), _p(ri))
    return (r,) if gauge == 0 else (d, ri)


def dip_block(rows, sym1, cols, sym2, q, compute, k, n_b, gauge, S, mats):
    """construct_dip_block_tensor for one pair of symmetries; mats as returned
    by setup_radial_dip."""
    rows, cols = np.ascontiguousarray(rows), np.ascontiguousarray(cols)
    S = np.asfortranarray(S, dtype=np.complex128)
    r = mats[0] if gauge == 0 else None
    d, ri = (mats[0], mats[1]) if gauge == 1 else (None, None)
    a = [_p(rows), rows.size, *[int(x) for x in sym1], _p(cols), cols.size,
         *[int(x) for x in sym2], int(q), int(bool(compute)), k, n_b, int(gauge), _p(S), _p(r),
         _p(d), _p(ri)]
    n = lib().or_dip_block(*a, None, None, None)
    D = dict(index_ptr=np.zeros(rows.size + 1, np.int64), indices=np.zeros(n, np.int64),
             data=np.zeros(n, np.complex128), nnz=n)
    lib().or_dip_block(*a, _p(D["index_ptr"]), _p(D["indices"]), _p(D["data"]))
    return D


def csr_mv(op, shape, index_ptr, indices, data, x):
    """CSR_mv (op 0), CSR_T_mv (op 1), CSR_mv_sym (op 2); returns (y, scale)."""
    ptr = np.ascontiguousarray(index_ptr, dtype=np.int64)
    idx = np.ascontiguousarray(indices, dtype=np.int64)
    dat = np.ascontiguousarray(data, dtype=np.complex128)
    xv = np.ascontiguousarray(x, dtype=np.complex128)
    n_out = shape[1] if op == 1 else shape[0]
    y = np.zeros(n_out, dtype=np.complex128)
    sc = np.zeros(n_out)
    lib().or_csr_mv(int(op), int(shape[0]), int(shape[1]), _p(ptr), _p(idx), _p(dat), _p(xv),
                    _p(y), _p(sc))
    return y, sc


def csr_from_blocks(blocks, n_rb, n_cb):
    """CSR_from_block of CSR dicts blocks[(i, j)]; returns one CSR dict."""
    order = [blocks[(i, j)] for j in range(n_cb) for i in range(n_rb)]
    nb = len(order)
    shapes = np.array([b["shape"] for b in order], dtype=np.int64).reshape(nb, 2)
    nnz = np.array([b["nnz"] for b in order], dtype=np.int64)
    P, I, D = (ctypes.c_void_p * nb)(), (ctypes.c_void_p * nb)(), (ctypes.c_void_p * nb)()
    keep = []
    for k, b in enumerate(order):
        if b["nnz"] > 0:
            arrs = (np.ascontiguousarray(b["index_ptr"], dtype=np.int64),
                    np.ascontiguousarray(b["indices"], dtype=np.int64),
                    np.ascontiguousarray(b["data"], dtype=np.complex128))
            keep.append(arrs)
            P[k], I[k], D[k] = (a.ctypes.data for a in arrs)
    rows = int(sum(shapes[i, 0] for i in range(n_rb)))
    tot = int(nnz.sum())
    out = dict(shape=(rows, int(sum(shapes[n_rb * j, 1] for j in range(n_cb)))), nnz=tot,
               index_ptr=np.zeros(rows + 1, np.int64), indices=np.zeros(tot, np.int64),
               data=np.zeros(tot, np.complex128))
    n = lib().or_csr_from_blocks(n_rb, n_cb, _p(shapes), _p(nnz), P, I, D, _p(out["index_ptr"]),
                                 _p(out["indices"]), _p(out["data"]))
    assert n == tot
    return out
