"""Mat-vec with the assembled blocks: CSR_mv, CSR_T_mv, CSR_mv_sym
(src/tools/sparse_array_tools.f90:966-1074).

The oracle's three products are pinned against dense numpy products on CPU;
the GPU products (through the C ABI) are compared with the oracle on blocks
the oracle assembles.  The GPU sums in another order (warp reduction, FP64
atomics), so the bar is |y_gpu - y_oracle| <= 1e-13 * sum |a_ij| |x_j|.
"""
import numpy as np
import pytest

from cases import CASES, blocks, oracle_reference

RTOL = 1e-13


def _dense(A):
    n, m = A["shape"]
    D = np.zeros((n, m), dtype=np.complex128)
    for i in range(n):
        for j in range(A["index_ptr"][i] - 1, A["index_ptr"][i + 1] - 1):
            D[i, A["indices"][j] - 1] += A["data"][j]
    return D


def _random_csr(rng, n, m, density, symmetric_upper=False):
    ptr, idx, dat = [1], [], []
    for i in range(n):
        cols = np.flatnonzero(rng.random(m) < density)
        if symmetric_upper:
            cols = cols[cols >= i]
        idx.extend(cols + 1)
        dat.extend(rng.standard_normal(cols.size) + 1j * rng.standard_normal(cols.size))
        ptr.append(len(idx) + 1)
    return dict(shape=(n, m), nnz=len(idx), index_ptr=np.array(ptr, np.int64),
                indices=np.array(idx, np.int64), data=np.array(dat, np.complex128))


@pytest.fixture(scope="module")
def small2_blocks(bs2e, oracle):
    """Oracle-assembled H (full and upper) and S of the small2 L=1 singlet block."""
    c = CASES["small2"]
    ref = oracle_reference("small2")
    (L, M, par, spin, cf) = [b for b in blocks(bs2e, "small2") if b[0] == 1 and b[3] == 0][0]
    out = {}
    for full in (True, False):
        H, S = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"], ref["H1p"],
                                      ref["S"], full, spin)
        H["shape"] = S["shape"] = (cf.size, cf.size)
        out["H_full" if full else "H_upper"] = H
        out["S_full" if full else "S_upper"] = S
    return out


@pytest.mark.parametrize("op", [0, 1, 2])
def test_oracle_products_match_dense(oracle, op):
    rng = np.random.default_rng(op)
    A = _random_csr(rng, 37, 37, 0.2)
    D = _dense(A)
    x = rng.standard_normal(37) + 1j * rng.standard_normal(37)
    y, sc = oracle.csr_mv(op, A["shape"], A["index_ptr"], A["indices"], A["data"], x)
    if op == 0:
        want = D @ x
    elif op == 1:
        want = D.T @ x
    else:
        U = np.triu(D)
        want = (U + np.triu(D, 1).T) @ x
    np.testing.assert_allclose(y, want, rtol=1e-13, atol=1e-13)
    assert (sc >= np.abs(y) * (1 - 1e-12)).all()


def test_oracle_rectangular_transpose(oracle):
    rng = np.random.default_rng(7)
    A = _random_csr(rng, 11, 23, 0.3)
    x = rng.standard_normal(11) + 1j * rng.standard_normal(11)
    y, _ = oracle.csr_mv(1, A["shape"], A["index_ptr"], A["indices"], A["data"], x)
    np.testing.assert_allclose(y, _dense(A).T @ x, rtol=1e-13, atol=1e-13)


def test_oracle_sym_equals_full_product_of_symmetric_block(oracle, small2_blocks):
    """CSR_mv_sym on the upper-stored block equals CSR_mv on the full block
    (the assembled H is complex symmetric)."""
    Hf, Hu = small2_blocks["H_full"], small2_blocks["H_upper"]
    rng = np.random.default_rng(3)
    x = rng.standard_normal(Hf["shape"][1]) + 1j * rng.standard_normal(Hf["shape"][1])
    yf, sf = oracle.csr_mv(0, Hf["shape"], Hf["index_ptr"], Hf["indices"], Hf["data"], x)
    yu, _ = oracle.csr_mv(2, Hu["shape"], Hu["index_ptr"], Hu["indices"], Hu["data"], x)
    assert (np.abs(yf - yu) <= 1e-12 * sf + 1e-300).all()


def _check(y, want, scale):
    err = np.abs(y - want)
    bound = RTOL * scale + 1e-300
    assert (err <= bound).all(), "max err/scale %g" % np.max(err / (scale + 1e-300))


@pytest.mark.gpu
@pytest.mark.parametrize("name,op", [("H_full", 0), ("H_full", 1), ("H_upper", 2),
                                     ("S_full", 0), ("S_upper", 2), ("H_upper", 0)])
def test_gpu_mv_matches_oracle(bs2e, oracle, small2_blocks, name, op):
    A = small2_blocks[name]
    n_in = A["shape"][0] if op == 1 else A["shape"][1]
    rng = np.random.default_rng(11 + op)
    x = rng.standard_normal(n_in) + 1j * rng.standard_normal(n_in)
    want, scale = oracle.csr_mv(op, A["shape"], A["index_ptr"], A["indices"], A["data"], x)
    c = CASES["small2"]
    with bs2e.Bs2e(oracle_reference("small2")["knots"], c["k"], c["q"], c["max_k"]) as h:
        y1 = h.csr_mv(A, x, op)
        y2 = h.csr_mv(A, x, op)  # buffers reused
    _check(y1, want, scale)
    _check(y2, want, scale)


@pytest.mark.gpu
@pytest.mark.parametrize("op", [0, 1, 2])
def test_gpu_mv_random_and_rectangular(bs2e, oracle, op):
    rng = np.random.default_rng(100 + op)
    shape = (300, 300) if op == 2 else (300, 170)
    A = _random_csr(rng, *shape, 0.05)
    A["data"][::7] = 0.0  # stored zeros stay stored
    n_in = shape[0] if op == 1 else shape[1]
    x = rng.standard_normal(n_in) + 1j * rng.standard_normal(n_in)
    want, scale = oracle.csr_mv(op, A["shape"], A["index_ptr"], A["indices"], A["data"], x)
    c = CASES["ref60"]
    with bs2e.Bs2e(oracle_reference("ref60")["knots"], c["k"], c["q"], c["max_k"]) as h:
        _check(h.csr_mv(A, x, op), want, scale)


@pytest.mark.gpu
def test_gpu_mv_on_device_blocks(bs2e, oracle):
    """Blocks filled into HBM (bs2e_block_fill_ex) multiplied in place."""
    torch = pytest.importorskip("torch")
    c = CASES["small2"]
    ref = oracle_reference("small2")
    (L, M, par, spin, cf) = [b for b in blocks(bs2e, "small2") if b[0] == 2 and b[3] == 1][0]
    Hr, _ = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"], ref["H1p"],
                                   ref["S"], True, spin)
    Hr["shape"] = (cf.size, cf.size)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(cf.size) + 1j * rng.standard_normal(cf.size)
    want, scale = oracle.csr_mv(0, Hr["shape"], Hr["index_ptr"], Hr["indices"], Hr["data"], x)
    dev = torch.device("cuda", 0)
    with bs2e.Bs2e(ref["knots"], c["k"], c["q"], c["max_k"]) as h:
        h.slater()
        h.rk()
        h.set_one_body(ref["H1p"], ref["S"])
        nH, nS = h.block_count(cf, L, True, spin)
        n = cf.size
        Hd = dict(index_ptr=torch.empty(n + 1, dtype=torch.int64, device=dev),
                  indices=torch.empty(nH, dtype=torch.int64, device=dev),
                  data=torch.empty(nH, dtype=torch.complex128, device=dev))
        Sd = dict(index_ptr=torch.empty(n + 1, dtype=torch.int64, device=dev),
                  indices=torch.empty(nS, dtype=torch.int64, device=dev),
                  data=torch.empty(nS, dtype=torch.complex128, device=dev))
        h.block_fill_into(cf, L, True, spin, {k: v.data_ptr() for k, v in Hd.items()},
                          {k: v.data_ptr() for k, v in Sd.items()}, on_device=True)
        xd = torch.from_numpy(x).to(dev)
        yd = torch.empty(n, dtype=torch.complex128, device=dev)
        torch.cuda.synchronize()  # x was copied on torch's stream; the library uses its own
        h.csr_mv_device(0, n, n, nH, Hd["index_ptr"].data_ptr(), Hd["indices"].data_ptr(),
                        Hd["data"].data_ptr(), xd.data_ptr(), yd.data_ptr())
        y = yd.cpu().numpy()
    _check(y, want, scale)


@pytest.mark.gpu
def test_gpu_mv_empty_and_errors(bs2e):
    c = CASES["ref60"]
    t = oracle_reference("ref60")["knots"]
    with bs2e.Bs2e(t, c["k"], c["q"], c["max_k"]) as h:
        E = dict(shape=(4, 3), nnz=0, index_ptr=np.ones(5, np.int64), indices=None, data=None)
        for op in (0, 1):
            y = h.csr_mv(E, np.ones(3 if op == 0 else 4, np.complex128), op)
            assert (y == 0).all()
        bad_col = dict(shape=(2, 2), nnz=2, index_ptr=np.array([1, 2, 3]),
                       indices=np.array([1, 3]), data=np.ones(2, np.complex128))
        with pytest.raises(bs2e.Bs2eError, match="column index"):
            h.csr_mv(bad_col, np.ones(2, np.complex128))
        bad_ptr = dict(shape=(2, 2), nnz=2, index_ptr=np.array([1, 9, 3]),
                       indices=np.array([1, 2]), data=np.ones(2, np.complex128))
        with pytest.raises(bs2e.Bs2eError, match="index_ptr"):
            h.csr_mv(bad_ptr, np.ones(2, np.complex128))
        with pytest.raises(bs2e.Bs2eError, match="square"):
            h.csr_mv(dict(shape=(2, 3), nnz=0, index_ptr=np.ones(3, np.int64)),
                     np.ones(3, np.complex128), op=2)
        # the handle stays usable after a rejected call
        ok = dict(shape=(2, 2), nnz=2, index_ptr=np.array([1, 2, 3]), indices=np.array([2, 1]),
                  data=np.array([2.0, 3.0 + 1j]))
        np.testing.assert_allclose(h.csr_mv(ok, np.array([1.0, 1j])), [2j, 3 + 1j])


@pytest.mark.gpu
def test_misaligned_device_pointers_rejected(bs2e):
    """Device pointers that break the 8/16-byte alignment of int64 / complex128
    arrays are refused on the host before any kernel runs."""
    torch = pytest.importorskip("torch")
    c = CASES["ref60"]
    dev = torch.device("cuda", 0)
    raw = torch.zeros(64, dtype=torch.float64, device=dev)
    p = raw.data_ptr()
    with bs2e.Bs2e(oracle_reference("ref60")["knots"], c["k"], c["q"], c["max_k"]) as h:
        with pytest.raises(bs2e.Bs2eError, match="align"):
            h.csr_mv_device(0, 2, 2, 2, p, p + 24, p + 8 * 9, p + 8 * 20, p + 8 * 30)
        # the handle stays usable
        ok = dict(shape=(1, 1), nnz=1, index_ptr=np.array([1, 2]), indices=np.array([1]),
                  data=np.array([2.0 + 0j]))
        np.testing.assert_allclose(h.csr_mv(ok, np.array([3.0 + 0j])), [6.0])


@pytest.mark.gpu
def test_gpu_mv_columns_8_byte_aligned(bs2e, oracle):
    """Column indices that start 8 bytes past a 16-byte boundary (valid: int64
    arrays need 8-byte alignment) take the vector path after one leading
    entry per row where needed; rows of every parity of start and length."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    A = _random_csr(rng, 200, 150, 0.07)
    x = rng.standard_normal(150) + 1j * rng.standard_normal(150)
    want, scale = oracle.csr_mv(0, A["shape"], A["index_ptr"], A["indices"], A["data"], x)
    dev = torch.device("cuda", 0)
    c = CASES["ref60"]
    with bs2e.Bs2e(oracle_reference("ref60")["knots"], c["k"], c["q"], c["max_k"]) as h:
        for shift in (0, 1):
            idx_buf = torch.zeros(A["nnz"] + 1, dtype=torch.int64, device=dev)
            idx = idx_buf[shift:shift + A["nnz"]]
            idx.copy_(torch.from_numpy(A["indices"]))
            assert (idx.data_ptr() % 16 == 0) == (shift == 0)
            ptr = torch.from_numpy(A["index_ptr"]).to(dev)
            dat = torch.from_numpy(A["data"]).to(dev)
            xd = torch.from_numpy(x).to(dev)
            yd = torch.empty(200, dtype=torch.complex128, device=dev)
            torch.cuda.synchronize()  # inputs copied on torch's stream
            h.csr_mv_device(0, 200, 150, A["nnz"], ptr.data_ptr(), idx.data_ptr(),
                            dat.data_ptr(), xd.data_ptr(), yd.data_ptr())
            _check(yd.cpu().numpy(), want, scale)


@pytest.mark.gpu
def test_stream_priority_keeps_products(bs2e, oracle):
    """bs2e_set_stream_priority recreates the handle's stream (a new stream,
    same products); priorities outside the device's range are refused and
    leave the handle usable."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    A = _random_csr(rng, 120, 90, 0.1)
    x = rng.standard_normal(90) + 1j * rng.standard_normal(90)
    want, scale = oracle.csr_mv(0, A["shape"], A["index_ptr"], A["indices"], A["data"], x)
    least, greatest = torch.cuda.Stream.priority_range()
    c = CASES["ref60"]
    with bs2e.Bs2e(oracle_reference("ref60")["knots"], c["k"], c["q"], c["max_k"]) as h:
        s0 = h.stream
        h.set_stream_priority(greatest)
        assert h.stream != s0
        _check(h.csr_mv(A, x, 0), want, scale)
        # torch's range may be narrower than the device's; these are outside both
        with pytest.raises(bs2e.Bs2eError, match="priority range"):
            h.set_stream_priority(-1000)
        with pytest.raises(bs2e.Bs2eError, match="priority range"):
            h.set_stream_priority(1000)
        h.set_stream_priority(least)
        _check(h.csr_mv(A, x, 0), want, scale)


@pytest.mark.gpu
def test_gpu_mv_long_rows_mixed_batches(bs2e, oracle):
    """y = A x on rows of 0..1500 entries: rows span many two-step batches,
    odd lengths start rows off the 16-byte boundary, complex entries sit in
    some batches only (the rest take the real-only branch), and a bad column
    deep inside a row is still caught."""
    rng = np.random.default_rng(31)
    n, m = 64, 4000
    ptr, idx, dat = [1], [], []
    for i in range(n):
        ln = int(rng.integers(0, 1500)) | (i & 1)  # odd lengths on odd rows
        cols = np.sort(rng.choice(m, size=ln, replace=False)) + 1
        vals = rng.standard_normal(ln).astype(np.complex128)
        if i % 3 == 0 and ln:
            k = rng.choice(ln, size=max(1, ln // 200), replace=False)
            vals[k] += 1j * rng.standard_normal(k.size)
        idx.extend(cols)
        dat.extend(vals)
        ptr.append(len(idx) + 1)
    A = dict(shape=(n, m), nnz=len(idx), index_ptr=np.array(ptr, np.int64),
             indices=np.array(idx, np.int64), data=np.array(dat, np.complex128))
    x = rng.standard_normal(m) + 1j * rng.standard_normal(m)
    want, scale = oracle.csr_mv(0, A["shape"], A["index_ptr"], A["indices"], A["data"], x)
    c = CASES["ref60"]
    with bs2e.Bs2e(oracle_reference("ref60")["knots"], c["k"], c["q"], c["max_k"]) as h:
        _check(h.csr_mv(A, x, 0), want, scale)
        bad = dict(A)
        bad["indices"] = A["indices"].copy()
        row = int(np.argmax(np.diff(A["index_ptr"])))
        bad["indices"][A["index_ptr"][row] - 1 + 700] = m + 1
        with pytest.raises(bs2e.Bs2eError, match="column index"):
            h.csr_mv(bad, x, 0)
        _check(h.csr_mv(A, x, 0), want, scale)  # still usable
