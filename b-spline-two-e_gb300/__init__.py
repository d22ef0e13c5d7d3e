"""GB300 two-electron matrix elements for B-spline bases (host-side mirror).

Python mirror of the interface that basis_setup uses in edvinolo/b-spline-two-e
(src/apps/main_basis_setup.f90:75-118) on top of the C-ABI CUDA library
libbs2e.so (include/bs2e.h).  The compute path is the CUDA library only: if
libbs2e.so cannot be loaded every call raises; nothing here falls back to a CPU
implementation.

Typical use, mirroring main_basis_setup.f90:
    h = Bs2e(knots, k, k_GL, max_k)          # splines%init + r_k/r_m_k/r_d_k%init
    h.slater()                               # setup_Slater_integrals
    h.rk()                                   # compute_R_k_map
    h.one_body(Z, n_l, ...)                  # setup_S / setup_H_one_particle
    for sym in symmetries(...):              # bas%init
        H, S = h.block(configs, sym.L, full)  # count_nnz + construct_block_tensor
"""
import ctypes
import os

import numpy as np

from . import grids, basis  # noqa: F401  (re-exported helpers)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbs2e.so")

PREC_FP64 = 0
PREC_MIXED = 1

_STATUS = {
    0: "BS2E_OK", 1: "BS2E_ERR_ARG", 2: "BS2E_ERR_NOMEM", 3: "BS2E_ERR_CUDA",
    4: "BS2E_ERR_COUNT", 5: "BS2E_ERR_TIMEOUT", 6: "BS2E_ERR_STATE", 7: "BS2E_ERR_NODEV",
    8: "BS2E_ERR_ORDER",
}

# Every symbol include/bs2e.h declares (checked by the CPU tests).
EXPORTS = [
    "bs2e_default_opts", "bs2e_create", "bs2e_destroy", "bs2e_last_error", "bs2e_sizes",
    "bs2e_slater", "bs2e_get_primitives", "bs2e_rk", "bs2e_rk_get", "bs2e_rk_get_batch",
    "bs2e_set_one_body", "bs2e_one_body", "bs2e_block_count", "bs2e_block_fill",
    "bs2e_block_count_ex", "bs2e_block_fill_ex", "bs2e_blocks_count_all",
    "bs2e_blocks_fill_all", "bs2e_configs", "bs2e_ang_k_LS",
    "bs2e_three_j", "bs2e_six_j", "bs2e_stream", "bs2e_set_stream_priority",
    "bs2e_launch_count", "bs2e_synchronize",
    "bs2e_radial_dipole", "bs2e_set_radial_dipole", "bs2e_dip_block_count", "bs2e_dip_block_fill",
    "bs2e_rk_get_batch_static", "bs2e_write_block_diag", "bs2e_write_block",
    "bs2e_csr_mv", "bs2e_block_count_rows", "bs2e_block_fill_rows", "bs2e_rk_export",
    "bs2e_batch_create", "bs2e_batch_run", "bs2e_batch_tuning", "bs2e_batch_destroy",
    "bs2e_csr_from_blocks", "bs2e_block_band_count", "bs2e_block_fill_band",
    "bs2e_set_block_cache", "bs2e_band_plan", "bs2e_band_rows", "bs2e_band_merge",
]


class Bs2eError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__("%s: %s" % (_STATUS.get(status, str(status)), msg))


class _Opts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int64), ("device", ctypes.c_int64),
                ("stage_bytes", ctypes.c_int64), ("reserved", ctypes.c_int64 * 5)]


_lib = None


def lib():
    """Loads libbs2e.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise Bs2eError(3, "libbs2e.so not built at %s (run build.py)" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    i64, p, dbl = ctypes.c_int64, ctypes.c_void_p, ctypes.c_double
    st = ctypes.c_int32
    sig = {
        "bs2e_default_opts": (None, [p]),
        "bs2e_create": (st, [p, i64, i64, i64, i64, p, p]),
        "bs2e_destroy": (st, [p]),
        "bs2e_last_error": (st, [p, p, i64]),
        "bs2e_sizes": (st, [p, p, p, p, p]),
        "bs2e_slater": (st, [p]),
        "bs2e_get_primitives": (st, [p, p, p, p, p, p]),
        "bs2e_rk": (st, [p, i64, i64]),
        "bs2e_rk_get": (st, [p, p, p]),
        "bs2e_rk_get_batch": (st, [p, i64, p, p]),
        "bs2e_rk_get_batch_static": (st, [p, i64, p, p]),
        "bs2e_write_block_diag": (st, [ctypes.c_char_p, i64, p, p, p, p, p, i64]),
        "bs2e_write_block": (st, [ctypes.c_char_p, i64, i64, p, p, p, p, p, i64]),
        "bs2e_csr_mv": (st, [p, i64, i64, i64, i64, p, p, p, p, p, i64]),
        "bs2e_rk_export": (st, [p, i64, p, i64]),
        "bs2e_batch_create": (st, [p, i64, p]),
        "bs2e_batch_run": (st, [p]),
        "bs2e_batch_tuning": (st, [p, p, p, p, p]),
        "bs2e_batch_destroy": (st, [p]),
        "bs2e_csr_from_blocks": (st, [p, i64, i64, p, p, p, p, p, p, p, p, i64]),
        "bs2e_block_count_rows": (st, [p, p, i64, i64, i64, i64, i64, i64, p, p]),
        "bs2e_block_fill_rows": (st, [p, p, i64, i64, i64, i64, i64, i64, p, p, p, p, p, p, i64]),
        "bs2e_block_band_count": (st, [p, p, i64, i64, i64, i64, i64, i64, p, p, p, p]),
        "bs2e_block_fill_band": (st, [p, p, i64, i64, i64, i64, i64, i64, p, p, p, p, p, p, p,
                                      i64]),
        "bs2e_set_block_cache": (st, [p, i64]),
        "bs2e_band_plan": (st, [i64, p, p, i64, i64, i64, p, p]),
        "bs2e_band_rows": (st, [p, i64, i64, i64, p, p]),
        "bs2e_band_merge": (st, [i64, i64, p, p, p, p, p, p, p, p]),
        "bs2e_set_one_body": (st, [p, p, i64, p]),
        "bs2e_one_body": (st, [p, i64, i64, i64, dbl, dbl, dbl, p, p]),
        "bs2e_block_count": (st, [p, p, i64, i64, i64, p, p]),
        "bs2e_block_fill": (st, [p, p, i64, i64, i64, p, i64, p, p, p, p, p, p, p]),
        "bs2e_block_count_ex": (st, [p, p, i64, i64, i64, i64, p, p]),
        "bs2e_block_fill_ex": (st, [p, p, i64, i64, i64, i64, p, p, p, p, p, p, i64]),
        "bs2e_blocks_count_all": (st, [p, i64, p, p, p, p, i64, p, p]),
        "bs2e_blocks_fill_all": (st, [p, i64, p, p, p, p, i64, p, p, p, p, p, p, i64]),
        "bs2e_configs": (st, [i64, i64, i64, i64, i64, i64, i64, i64, i64, p, p]),
        "bs2e_ang_k_LS": (dbl, [i64, i64, i64, i64, i64, i64]),
        "bs2e_three_j": (dbl, [i64, i64, i64, i64, i64, i64]),
        "bs2e_six_j": (dbl, [i64, i64, i64, i64, i64, i64]),
        "bs2e_stream": (st, [p, p]),
        "bs2e_set_stream_priority": (st, [p, i64]),
        "bs2e_launch_count": (st, [p, p]),
        "bs2e_synchronize": (st, [p]),
        "bs2e_radial_dipole": (st, [p, i64, p, p, p]),
        "bs2e_set_radial_dipole": (st, [p, i64, p, p, p]),
        "bs2e_dip_block_count": (st, [p, p, i64, i64, i64, i64, p, i64, i64, i64, i64, i64, i64,
                                      p]),
        "bs2e_dip_block_fill": (st, [p, p, i64, i64, i64, i64, p, i64, i64, i64, i64, i64, i64,
                                     p, p, p, i64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


CONFIG_DTYPE = np.dtype([("n1", "<i8"), ("n2", "<i8"), ("l1", "<i8"), ("l2", "<i8"),
                         ("eqv", "<i8")])


def as_configs(cf):
    """Configuration list as a contiguous int64 record array (n1, n2, l1, l2, eqv)."""
    a = np.asarray(cf)
    if a.dtype == CONFIG_DTYPE:
        return np.ascontiguousarray(a)
    a = np.ascontiguousarray(a, dtype=np.int64).reshape(-1, 5)
    return a.view(CONFIG_DTYPE).reshape(-1)


def configs(L, parity_odd, max_l_1p, n_b, k, max_n_b=None, n_all_l=None, l2_max=None, spin=0):
    """count_configs (src/tools/orbital_tools.f90:119-216) through the library."""
    L_ = lib()
    max_n_b = n_b if max_n_b is None else max_n_b
    n_all_l = n_b if n_all_l is None else n_all_l
    l2_max = max_l_1p if l2_max is None else l2_max
    n = ctypes.c_int64()
    args = [L, int(parity_odd), max_l_1p, n_b, k, max_n_b, n_all_l, l2_max, spin]
    _check(None, L_.bs2e_configs(*args, None, ctypes.byref(n)))
    out = np.zeros(n.value, dtype=CONFIG_DTYPE)
    _check(None, L_.bs2e_configs(*args, _ptr(out), ctypes.byref(n)))
    return out


def ang_k_LS(k, la, lb, lc, ld, L):
    return lib().bs2e_ang_k_LS(k, la, lb, lc, ld, L)


def three_j(ja, jb, jc, ma, mb, mc):
    return lib().bs2e_three_j(ja, jb, jc, ma, mb, mc)


def six_j(ja, jb, jc, jd, je, jf):
    return lib().bs2e_six_j(ja, jb, jc, jd, je, jf)


def _block_arrays(blocks):
    n = len(blocks)
    shapes = np.zeros((n, 2), dtype=np.int64)
    nnz = np.zeros(n, dtype=np.int64)
    P = (ctypes.c_void_p * max(n, 1))()
    I = (ctypes.c_void_p * max(n, 1))()
    D = (ctypes.c_void_p * max(n, 1))()
    keep = []
    for i, b in enumerate(blocks):
        shapes[i] = b["shape"]
        nnz[i] = b["nnz"]
        if b["nnz"] > 0:
            arrs = (np.ascontiguousarray(b["index_ptr"], dtype=np.int64),
                    np.ascontiguousarray(b["indices"], dtype=np.int64),
                    np.ascontiguousarray(b["data"], dtype=np.complex128))
            keep.append(arrs)
            P[i], I[i], D[i] = (a.ctypes.data for a in arrs)
    return shapes, nnz, P, I, D, keep


def write_block_diag(path, blocks, max_subrecord=0):
    """H_diag.dat / S_diag.dat (CS_block_diag_store, block_tools.f90:458-485):
    blocks is a list of dicts with shape, nnz, index_ptr, indices, data."""
    shapes, nnz, P, I, D, keep = _block_arrays(blocks)
    _check(None, lib().bs2e_write_block_diag(os.fsencode(path), len(blocks), _ptr(shapes),
                                             _ptr(nnz), P, I, D, int(max_subrecord)))


def write_block(path, blocks, n_rows_b, n_cols_b, max_subrecord=0):
    """D_q.dat (CS_block_store, block_tools.f90:386-415): blocks[(i, j)]."""
    order = [blocks[(i, j)] for j in range(n_cols_b) for i in range(n_rows_b)]
    shapes, nnz, P, I, D, keep = _block_arrays(order)
    _check(None, lib().bs2e_write_block(os.fsencode(path), n_rows_b, n_cols_b, _ptr(shapes),
                                        _ptr(nnz), P, I, D, int(max_subrecord)))


def band_plan(per_n1, max_bytes, n_ranks=1):
    """Bands of every block that fit max_bytes, each with its owner rank
    (bs2e_band_plan): per_n1[b] is block b's (n1_max, 3) array of (rows,
    nnz_H, nnz_S) per n1.  Returns an (n_bands, 5) array of (block, n1_first,
    n1_count, owner, bytes)."""
    per = [np.ascontiguousarray(p, dtype=np.int64) for p in per_n1]
    nmax = np.array([p.shape[0] for p in per], dtype=np.int64)
    ptrs = (ctypes.c_void_p * max(len(per), 1))(*[p.ctypes.data for p in per])
    n = ctypes.c_int64()
    st = lib().bs2e_band_plan(len(per), _ptr(nmax), ptrs, int(max_bytes), int(n_ranks), 0, None,
                              ctypes.byref(n))
    if st != 0 and n.value == 0:
        _check(None, st)
    out = np.zeros((max(n.value, 1), 5), dtype=np.int64)
    _check(None, lib().bs2e_band_plan(len(per), _ptr(nmax), ptrs, int(max_bytes), int(n_ranks),
                                      n.value, _ptr(out), ctypes.byref(n)))
    return out[:n.value]


def band_rows(cf, n1_first, n1_count):
    """1-based block rows of an n1 band (bs2e_band_rows)."""
    cf = as_configs(cf)
    n = ctypes.c_int64()
    _check(None, lib().bs2e_band_rows(_ptr(cf), cf.size, int(n1_first), int(n1_count), None,
                                      ctypes.byref(n)))
    rows = np.zeros(max(n.value, 1), dtype=np.int64)
    _check(None, lib().bs2e_band_rows(_ptr(cf), cf.size, int(n1_first), int(n1_count),
                                      _ptr(rows), ctypes.byref(n)))
    return rows[:n.value]


def band_merge(n_config, bands):
    """Joins band CSRs into the block CSR (bs2e_band_merge): bands is a list
    of dicts with 'rows' (1-based block rows), 'index_ptr', 'indices', 'data'."""
    nb = len(bands)
    arr = lambda xs, t: (ctypes.c_void_p * max(nb, 1))(*[x.ctypes.data for x in xs])
    rows = [np.ascontiguousarray(b["rows"], dtype=np.int64) for b in bands]
    ptr = [np.ascontiguousarray(b["index_ptr"], dtype=np.int64) for b in bands]
    idx = [np.ascontiguousarray(b["indices"], dtype=np.int64) for b in bands]
    dat = [np.ascontiguousarray(b["data"], dtype=np.complex128) for b in bands]
    nrows = np.array([r.size for r in rows], dtype=np.int64)
    nnz = int(sum(int(p[-1]) - 1 for p in ptr))
    out = dict(index_ptr=np.zeros(n_config + 1, np.int64), indices=np.zeros(max(nnz, 1), np.int64),
               data=np.zeros(max(nnz, 1), np.complex128))
    _check(None, lib().bs2e_band_merge(int(n_config), nb, _ptr(nrows), arr(rows, 0), arr(ptr, 0),
                                       arr(idx, 0), arr(dat, 0), _ptr(out["index_ptr"]),
                                       _ptr(out["indices"]), _ptr(out["data"])))
    out["indices"] = out["indices"][:nnz]
    out["data"] = out["data"][:nnz]
    out["nnz"] = nnz
    return out


def _check(h, status):
    if status != 0:
        msg = ""
        if h is not None:
            buf = ctypes.create_string_buffer(1024)
            lib().bs2e_last_error(h, buf, 1024)
            msg = buf.value.decode(errors="replace")
        raise Bs2eError(status, msg)


class Bs2e:
    """One B-spline basis on one GPU (wraps a bs2e_handle)."""

    def __init__(self, knots, k, k_GL, max_k, precision=PREC_FP64, device=0, stage_bytes=0):
        L_ = lib()
        self.knots = np.ascontiguousarray(knots, dtype=np.float64)
        self.k, self.k_GL, self.max_k = int(k), int(k_GL), int(max_k)
        self.K1 = self.max_k + 1
        self.precision = int(precision)
        opts = _Opts()
        L_.bs2e_default_opts(ctypes.byref(opts))
        opts.precision = int(precision)
        opts.device = int(device)
        opts.stage_bytes = int(stage_bytes)
        h = ctypes.c_void_p()
        st = L_.bs2e_create(_ptr(self.knots), self.knots.size, self.k, self.k_GL, self.max_k,
                            ctypes.byref(opts), ctypes.byref(h))
        if st != 0:
            raise Bs2eError(st, "bs2e_create failed")
        self._h = h
        nb, niv, n4, n6 = (ctypes.c_int64() for _ in range(4))
        _check(h, L_.bs2e_sizes(h, *(ctypes.byref(x) for x in (nb, niv, n4, n6))))
        self.n_b, self.n_iv, self.nnz4, self.nnz6 = nb.value, niv.value, n4.value, n6.value

    def close(self):
        if getattr(self, "_h", None):
            lib().bs2e_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- radial stage --------------------------------------------------------
    def slater(self):
        _check(self._h, lib().bs2e_slater(self._h))

    def primitives(self, with_diag=True):
        """r_k, r_m_k (nnz4 x K1), idx4 (nnz4 x 3), r_d_k (nnz6 x K1), idx6 (nnz6 x 5)."""
        rk = np.zeros((self.nnz4, self.K1), order="F")
        rmk = np.zeros((self.nnz4, self.K1), order="F")
        i4 = np.zeros((self.nnz4, 3), dtype=np.int64)
        rdk = i6 = None
        if with_diag:
            rdk = np.zeros((self.nnz6, self.K1), order="F")
            i6 = np.zeros((self.nnz6, 5), dtype=np.int64)
        _check(self._h, lib().bs2e_get_primitives(self._h, _ptr(rk), _ptr(rmk), _ptr(i4),
                                                  _ptr(rdk), _ptr(i6)))
        return dict(r_k=rk, r_m_k=rmk, idx4=i4, r_d_k=rdk, idx6=i6)

    def rk(self, k_first=0, k_count=None):
        k_count = self.K1 - k_first if k_count is None else k_count
        _check(self._h, lib().bs2e_rk(self._h, k_first, k_count))

    def rk_get(self, keys):
        """R^k values (n x K1) of 1-based keys [a,b,c,d] (n x 4)."""
        keys = np.ascontiguousarray(keys, dtype=np.int64).reshape(-1, 4)
        vals = np.zeros((keys.shape[0], self.K1))
        _check(self._h, lib().bs2e_rk_get_batch(self._h, keys.shape[0], _ptr(keys), _ptr(vals)))
        return vals

    def rk_get_static(self, keys):
        """rk_get through the allocation-free entry point (at most 4096 keys;
        see bs2e_rk_get_batch_static in include/bs2e.h)."""
        keys = np.ascontiguousarray(keys, dtype=np.int64).reshape(-1, 4)
        vals = np.zeros((keys.shape[0], self.K1))
        _check(self._h, lib().bs2e_rk_get_batch_static(self._h, keys.shape[0], _ptr(keys),
                                                       _ptr(vals)))
        return vals

    # -- one-body matrices ---------------------------------------------------
    def one_body(self, Z, n_l, cap_order=2, cap_r0=10.0, cap_eta=1e-3 + 0j, copy_out=True):
        H = S = None
        if copy_out:
            H = np.zeros((self.n_b, self.n_b, n_l), dtype=np.complex128, order="F")
            S = np.zeros((self.n_b, self.n_b), dtype=np.complex128, order="F")
        eta = complex(cap_eta)
        _check(self._h, lib().bs2e_one_body(self._h, int(Z), int(n_l), int(cap_order),
                                            float(cap_r0), eta.real, eta.imag, _ptr(H), _ptr(S)))
        return H, S

    def set_one_body(self, H1p, S):
        H1p = np.asfortranarray(H1p, dtype=np.complex128)
        S = np.asfortranarray(S, dtype=np.complex128)
        n_l = H1p.shape[2] if H1p.ndim == 3 else 1
        _check(self._h, lib().bs2e_set_one_body(self._h, _ptr(H1p), n_l, _ptr(S)))

    # -- symmetry blocks -------------------------------------------------------
    def block_count(self, cf, L, full=True, spin=0):
        cf = as_configs(cf)
        nh, ns = ctypes.c_int64(), ctypes.c_int64()
        _check(self._h, lib().bs2e_block_count_ex(self._h, _ptr(cf), cf.size, int(L), int(spin),
                                                  int(bool(full)), ctypes.byref(nh),
                                                  ctypes.byref(ns)))
        return nh.value, ns.value

    def block(self, cf, L, full=True, spin=0):
        """count + fill into host arrays; returns (H, S) dicts of 1-based CSR arrays."""
        cf = as_configs(cf)
        nh, ns = self.block_count(cf, L, full, spin)
        n = cf.size
        H = dict(shape=(n, n), nnz=nh, index_ptr=np.zeros(n + 1, np.int64),
                 indices=np.zeros(nh, np.int64), data=np.zeros(nh, np.complex128))
        S = dict(shape=(n, n), nnz=ns, index_ptr=np.zeros(n + 1, np.int64),
                 indices=np.zeros(ns, np.int64), data=np.zeros(ns, np.complex128))
        self.block_fill_into(cf, L, full, spin, H, S, on_device=False)
        return H, S

    def block_rows(self, cf, L, row_first, row_count, full=True, spin=0):
        """Rows [row_first, row_first + row_count) of a block into host arrays:
        (H, S) dicts with a range-local 1-based index_ptr."""
        cf = as_configs(cf)
        nh, ns = ctypes.c_int64(), ctypes.c_int64()
        a = [self._h, _ptr(cf), cf.size, int(L), int(spin), int(bool(full)), int(row_first),
             int(row_count)]
        _check(self._h, lib().bs2e_block_count_rows(*a, ctypes.byref(nh), ctypes.byref(ns)))
        n = int(row_count)
        H = dict(shape=(n, cf.size), nnz=nh.value, index_ptr=np.zeros(n + 1, np.int64),
                 indices=np.zeros(nh.value, np.int64), data=np.zeros(nh.value, np.complex128))
        S = dict(shape=(n, cf.size), nnz=ns.value, index_ptr=np.zeros(n + 1, np.int64),
                 indices=np.zeros(ns.value, np.int64), data=np.zeros(ns.value, np.complex128))
        _check(self._h, lib().bs2e_block_fill_rows(*a, *[_ptr(H[x]) for x in
                                                         ("index_ptr", "indices", "data")],
                                                   *[_ptr(S[x]) for x in
                                                     ("index_ptr", "indices", "data")], 0))
        return H, S

    def block_rows_into(self, cf, L, row_first, row_count, full, spin, H, S):
        """Rows of a block into device buffers (dicts of integer device addresses)."""
        cf = as_configs(cf)
        args = [ctypes.c_void_p(int(H[x])) for x in ("index_ptr", "indices", "data")]
        args += [ctypes.c_void_p(int(S[x])) for x in ("index_ptr", "indices", "data")]
        _check(self._h, lib().bs2e_block_fill_rows(self._h, _ptr(cf), cf.size, int(L), int(spin),
                                                   int(bool(full)), int(row_first),
                                                   int(row_count), *args, 1))

    def block_count_rows(self, cf, L, row_first, row_count, full=True, spin=0):
        cf = as_configs(cf)
        nh, ns = ctypes.c_int64(), ctypes.c_int64()
        _check(self._h, lib().bs2e_block_count_rows(self._h, _ptr(cf), cf.size, int(L),
                                                    int(spin), int(bool(full)), int(row_first),
                                                    int(row_count), ctypes.byref(nh),
                                                    ctypes.byref(ns)))
        return nh.value, ns.value

    def band_count(self, cf, L, n1_first, n1_count, full=True, spin=0, per_n1=False):
        """(rows, nnz_H, nnz_S) of the n1 band [n1_first, n1_first + n1_count)
        of a block; with per_n1 also an (n1_count, 3) array of the same per n1."""
        cf = as_configs(cf)
        r, nh, ns = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        per = np.zeros((int(n1_count), 3), dtype=np.int64) if per_n1 else None
        _check(self._h, lib().bs2e_block_band_count(self._h, _ptr(cf), cf.size, int(L), int(spin),
                                                    int(bool(full)), int(n1_first), int(n1_count),
                                                    ctypes.byref(r), ctypes.byref(nh),
                                                    ctypes.byref(ns), _ptr(per)))
        return (r.value, nh.value, ns.value, per) if per_n1 else (r.value, nh.value, ns.value)

    def band_into(self, cf, L, n1_first, n1_count, full, spin, H, S, rows=None):
        """Band fill into device buffers (dicts of integer device addresses;
        rows: device address for the 1-based block rows, or None)."""
        cf = as_configs(cf)
        args = [ctypes.c_void_p(int(H[x])) for x in ("index_ptr", "indices", "data")]
        args += [ctypes.c_void_p(int(S[x])) for x in ("index_ptr", "indices", "data")]
        rp = ctypes.c_void_p(int(rows)) if rows else None
        _check(self._h, lib().bs2e_block_fill_band(self._h, _ptr(cf), cf.size, int(L), int(spin),
                                                   int(bool(full)), int(n1_first), int(n1_count),
                                                   rp, *args, 1))

    def band_host_into(self, cf, L, n1_first, n1_count, full, spin, H, S, rows=None):
        """Band fill into host numpy arrays (dicts 'index_ptr', 'indices',
        'data'; rows: int64 array or None), staged through HBM."""
        cf = as_configs(cf)
        args = [_ptr(H[x]) for x in ("index_ptr", "indices", "data")]
        args += [_ptr(S[x]) for x in ("index_ptr", "indices", "data")]
        _check(self._h, lib().bs2e_block_fill_band(self._h, _ptr(cf), cf.size, int(L), int(spin),
                                                   int(bool(full)), int(n1_first), int(n1_count),
                                                   _ptr(rows), *args, 0))

    def band(self, cf, L, n1_first, n1_count, full=True, spin=0):
        """(rows, H, S) of an n1 band in host arrays."""
        r, nh, ns = self.band_count(cf, L, n1_first, n1_count, full, spin)
        mk = lambda n, m: dict(index_ptr=np.zeros(n + 1, np.int64),
                               indices=np.zeros(max(m, 1), np.int64),
                               data=np.zeros(max(m, 1), np.complex128), nnz=m)
        H, S, rows = mk(r, nh), mk(r, ns), np.zeros(max(r, 1), np.int64)
        self.band_host_into(cf, L, n1_first, n1_count, full, spin, H, S, rows)
        for M, m in ((H, nh), (S, ns)):
            M["indices"], M["data"] = M["indices"][:m], M["data"][:m]
        return rows[:r], H, S

    def set_block_cache(self, n_blocks):
        """Counted blocks kept besides the current one (0..16)."""
        _check(self._h, lib().bs2e_set_block_cache(self._h, int(n_blocks)))

    def block_fill_into(self, cf, L, full, spin, H, S, on_device=False):
        """Fills caller-provided arrays: numpy (host) or, with on_device, integer
        device addresses in the dicts' 'index_ptr', 'indices', 'data' entries."""
        cf = as_configs(cf)
        if on_device:
            args = [ctypes.c_void_p(int(H[x])) for x in ("index_ptr", "indices", "data")]
            args += [ctypes.c_void_p(int(S[x])) for x in ("index_ptr", "indices", "data")]
        else:
            args = [_ptr(H[x]) for x in ("index_ptr", "indices", "data")]
            args += [_ptr(S[x]) for x in ("index_ptr", "indices", "data")]
        _check(self._h, lib().bs2e_block_fill_ex(self._h, _ptr(cf), cf.size, int(L), int(spin),
                                                 int(bool(full)), *args, int(bool(on_device))))

    # -- all symmetry blocks in one call ---------------------------------------
    @staticmethod
    def _blocks_args(blocks):
        cfs = [as_configs(cf) for (cf, L, spin) in blocks]
        n = len(cfs)
        ptrs = (ctypes.c_void_p * max(n, 1))(*[cf.ctypes.data for cf in cfs])
        n_config = np.array([cf.size for cf in cfs], dtype=np.int64)
        Ls = np.array([int(L) for (_, L, _) in blocks], dtype=np.int64)
        spins = np.array([int(sp) for (_, _, sp) in blocks], dtype=np.int64)
        return cfs, ptrs, n_config, Ls, spins

    def blocks_count_all(self, blocks, full=True):
        """bs2e_blocks_count_all over blocks = [(configs, L, spin), ...];
        returns (nnz_H, nnz_S) int64 arrays."""
        cfs, ptrs, n_config, Ls, spins = self._blocks_args(blocks)
        nH = np.zeros(len(cfs), dtype=np.int64)
        nS = np.zeros(len(cfs), dtype=np.int64)
        _check(self._h, lib().bs2e_blocks_count_all(self._h, len(cfs), ptrs, _ptr(n_config),
                                                    _ptr(Ls), _ptr(spins), int(bool(full)),
                                                    _ptr(nH), _ptr(nS)))
        return nH, nS

    def blocks_fill_all_into(self, blocks, full, Hs, Ss, on_device=False):
        """bs2e_blocks_fill_all into caller arrays: Hs[i], Ss[i] are dicts as in
        block_fill_into (numpy arrays, or device addresses with on_device)."""
        cfs, ptrs, n_config, Ls, spins = self._blocks_args(blocks)
        n = max(len(cfs), 1)
        addr = (lambda v: int(v)) if on_device else (lambda v: v.ctypes.data)
        arr = lambda D, x: (ctypes.c_void_p * n)(*[addr(d[x]) for d in D])
        _check(self._h, lib().bs2e_blocks_fill_all(
            self._h, len(cfs), ptrs, _ptr(n_config), _ptr(Ls), _ptr(spins), int(bool(full)),
            arr(Hs, "index_ptr"), arr(Hs, "indices"), arr(Hs, "data"),
            arr(Ss, "index_ptr"), arr(Ss, "indices"), arr(Ss, "data"), int(bool(on_device))))

    def blocks_all(self, blocks, full=True):
        """Count and fill every block into host arrays; returns [(H, S), ...]."""
        nH, nS = self.blocks_count_all(blocks, full)
        Hs, Ss = [], []
        for (cf, L, spin), h, s in zip(blocks, nH, nS):
            n = as_configs(cf).size
            Hs.append(dict(shape=(n, n), nnz=int(h), index_ptr=np.zeros(n + 1, np.int64),
                           indices=np.zeros(h, np.int64), data=np.zeros(h, np.complex128)))
            Ss.append(dict(shape=(n, n), nnz=int(s), index_ptr=np.zeros(n + 1, np.int64),
                           indices=np.zeros(s, np.int64), data=np.zeros(s, np.complex128)))
        self.blocks_fill_all_into(blocks, full, Hs, Ss)
        return list(zip(Hs, Ss))

    # -- dipoles ---------------------------------------------------------------
    def radial_dipole(self, gauge=0, copy_out=True):
        """setup_radial_dip on the device; gauge 0 = length (returns r_mat),
        1 = velocity (returns dr_mat, r_inv_mat)."""
        mk = lambda: np.zeros((self.n_b, self.n_b), dtype=np.complex128, order="F")
        a = mk() if copy_out and gauge == 0 else None
        b = mk() if copy_out and gauge == 1 else None
        c = mk() if copy_out and gauge == 1 else None
        _check(self._h, lib().bs2e_radial_dipole(self._h, int(gauge), _ptr(a), _ptr(b), _ptr(c)))
        return (a,) if gauge == 0 else (b, c)

    def set_radial_dipole(self, gauge, r_mat=None, dr_mat=None, r_inv_mat=None):
        f = lambda m: None if m is None else np.asfortranarray(m, dtype=np.complex128)
        r_mat, dr_mat, r_inv_mat = f(r_mat), f(dr_mat), f(r_inv_mat)
        _check(self._h, lib().bs2e_set_radial_dipole(self._h, int(gauge), _ptr(r_mat),
                                                     _ptr(dr_mat), _ptr(r_inv_mat)))

    def dip_block_count(self, rows, sym1, cols, sym2, q, compute=True):
        """Non-zeros of a dipole block (count pass only)."""
        rows, cols = as_configs(rows), as_configs(cols)
        n = ctypes.c_int64()
        _check(self._h, lib().bs2e_dip_block_count(self._h, _ptr(rows), rows.size,
                                                   *[int(x) for x in sym1], _ptr(cols), cols.size,
                                                   *[int(x) for x in sym2], int(q),
                                                   int(bool(compute)), ctypes.byref(n)))
        return n.value

    def dip_block_into(self, rows, sym1, cols, sym2, q, D, compute=True):
        """Dipole block fill into device buffers: D holds integer device
        addresses under 'index_ptr', 'indices', 'data' (sized by dip_block_count)."""
        rows, cols = as_configs(rows), as_configs(cols)
        _check(self._h, lib().bs2e_dip_block_fill(
            self._h, _ptr(rows), rows.size, *[int(x) for x in sym1], _ptr(cols), cols.size,
            *[int(x) for x in sym2], int(q), int(bool(compute)),
            *[ctypes.c_void_p(int(D[x])) for x in ("index_ptr", "indices", "data")], 1))

    def dip_block(self, rows, sym1, cols, sym2, q, compute=True):
        """Dipole block between symmetries sym1 = (L1, M1, parity1) (rows) and
        sym2 = (L2, M2, parity2) (columns); returns a dict of 1-based CSR arrays."""
        rows, cols = as_configs(rows), as_configs(cols)
        a = [_ptr(rows), rows.size, *[int(x) for x in sym1], _ptr(cols), cols.size,
             *[int(x) for x in sym2], int(q), int(bool(compute))]
        n = ctypes.c_int64()
        _check(self._h, lib().bs2e_dip_block_count(self._h, *a, ctypes.byref(n)))
        D = dict(shape=(rows.size, cols.size), nnz=n.value,
                 index_ptr=np.zeros(rows.size + 1, np.int64), indices=np.zeros(n.value, np.int64),
                 data=np.zeros(n.value, np.complex128))
        _check(self._h, lib().bs2e_dip_block_fill(self._h, *a, _ptr(D["index_ptr"]),
                                                  _ptr(D["indices"]), _ptr(D["data"]), 0))
        return D

    def rk_export(self, k, out=None, on_device=False):
        """Multipole k of the store as an (N, N, W, W) array (host), or into the
        device address `out` with on_device."""
        W = 2 * self.k - 1
        if on_device:
            _check(self._h, lib().bs2e_rk_export(self._h, int(k), ctypes.c_void_p(int(out)), 1))
            return out
        if out is None:
            out = np.zeros((self.n_b, self.n_b, W, W))
        _check(self._h, lib().bs2e_rk_export(self._h, int(k), _ptr(out), 0))
        return out

    # -- mat-vec -------------------------------------------------------------
    def csr_mv(self, A, x, op=0, y=None):
        """CSR_mv (op 0), CSR_T_mv (op 1) or CSR_mv_sym (op 2) of a CSR dict
        (shape, nnz, index_ptr, indices, data) with x (host arrays)."""
        n_rows, n_cols = A["shape"]
        nnz = int(A["nnz"])
        ptr = np.ascontiguousarray(A["index_ptr"], dtype=np.int64)
        idx = np.ascontiguousarray(A["indices"], dtype=np.int64) if nnz else None
        dat = np.ascontiguousarray(A["data"], dtype=np.complex128) if nnz else None
        xv = np.ascontiguousarray(x, dtype=np.complex128)
        n_in, n_out = (n_rows, n_cols) if op == 1 else (n_cols, n_rows)
        if xv.size != n_in:
            raise ValueError("x has %d entries, the product needs %d" % (xv.size, n_in))
        if y is None:
            y = np.zeros(n_out, dtype=np.complex128)
        _check(self._h, lib().bs2e_csr_mv(self._h, int(op), n_rows, n_cols, nnz, _ptr(ptr),
                                          _ptr(idx), _ptr(dat), _ptr(xv), _ptr(y), 0))
        return y

    def csr_from_blocks(self, blocks, n_rb, n_cb):
        """CSR_from_block of host CSR dicts blocks[(i, j)] (shape, nnz and,
        when nnz > 0, index_ptr / indices / data); returns one CSR dict."""
        order = [blocks[(i, j)] for j in range(n_cb) for i in range(n_rb)]
        shapes, nnz, P, I, D, keep = _block_arrays(order)
        rows = sum(int(blocks[(i, 0)]["shape"][0]) for i in range(n_rb))
        cols = sum(int(blocks[(0, j)]["shape"][1]) for j in range(n_cb))
        tot = int(nnz.sum())
        out = dict(shape=(rows, cols), nnz=tot, index_ptr=np.zeros(rows + 1, np.int64),
                   indices=np.zeros(tot, np.int64), data=np.zeros(tot, np.complex128))
        _check(self._h, lib().bs2e_csr_from_blocks(self._h, n_rb, n_cb, _ptr(shapes), _ptr(nnz),
                                                   P, I, D, _ptr(out["index_ptr"]),
                                                   _ptr(out["indices"]), _ptr(out["data"]), 0))
        return out

    def csr_from_block_diag(self, blocks):
        """CSR_from_block_diag: the diagonal blocks joined into one CSR."""
        n = len(blocks)
        grid = {}
        for i in range(n):
            for j in range(n):
                grid[(i, j)] = blocks[i] if i == j else dict(
                    shape=(blocks[i]["shape"][0], blocks[j]["shape"][1]), nnz=0)
        return self.csr_from_blocks(grid, n, n)

    def csr_mv_device(self, op, n_rows, n_cols, nnz, ptr, idx, data, x, y):
        """The same product on device pointers (ints), e.g. torch tensors' data_ptr()."""
        _check(self._h, lib().bs2e_csr_mv(self._h, int(op), n_rows, n_cols, nnz, ptr, idx, data,
                                          x, y, 1))

    # -- plumbing ------------------------------------------------------------
    @property
    def stream(self):
        s = ctypes.c_void_p()
        _check(self._h, lib().bs2e_stream(self._h, ctypes.byref(s)))
        return s.value

    def set_stream_priority(self, priority):
        """Recreate the handle's stream with this CUDA stream priority (smaller
        is higher; see torch.cuda.Stream.priority_range())."""
        _check(self._h, lib().bs2e_set_stream_priority(self._h, int(priority)))

    @property
    def launch_count(self):
        c = ctypes.c_int64()
        _check(self._h, lib().bs2e_launch_count(self._h, ctypes.byref(c)))
        return c.value

    def synchronize(self):
        _check(self._h, lib().bs2e_synchronize(self._h))


class RadialBatch:
    """bs2e_slater + bs2e_rk of many Bs2e handles as one batched, graph-captured
    radial stage (bs2e_batch_*).  The handles must outlive the batch."""

    def __init__(self, handles):
        self.handles = list(handles)
        arr = (ctypes.c_void_p * len(self.handles))(*[h._h.value for h in self.handles])
        b = ctypes.c_void_p()
        _check(self.handles[0]._h, lib().bs2e_batch_create(arr, len(self.handles), ctypes.byref(b)))
        self._b = b

    def run(self):
        _check(self.handles[0]._h, lib().bs2e_batch_run(self._b))

    def tuning(self):
        v = [ctypes.c_int64() for _ in range(4)]
        lib().bs2e_batch_tuning(self._b, *[ctypes.byref(x) for x in v])
        return dict(rk_threads=v[0].value, chunk=v[1].value, graph=bool(v[2].value),
                    launches=v[3].value)

    def close(self):
        if getattr(self, "_b", None):
            lib().bs2e_batch_destroy(self._b)
            self._b = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()
