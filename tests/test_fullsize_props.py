"""Size-independent properties at the full size of the order-7, N=200 bench
workload (exp-linear knots to r_max=200, 10 GL points, k=0..10, l_max=5,
L=0..3 natural parity, singlet and triplet), where the oracle cannot rebuild
whole blocks in test time:

- every block's row count and H/S non-zero counts equal the oracle's
  count_nnz (tests/golden/order7_n200_counts.json, made by
  tests/golden/gen_fullsize_counts.py): bit-exact;
- the R^k store has the symmetries of the Slater integral,
  R[a,b,c,d] = R[c,b,a,d] = R[a,d,c,b] = R[b,a,d,c], and is positive wherever
  both pairs overlap (B-splines are non-negative);
- without the absorbing potential (eta = 0) H is real symmetric: H x = H^T x
  for a random x, and the symmetric product of the upper-triangle block
  (full = false, CSR_mv_sym semantics) equals the full block's product, all
  within 1e-12 of sum |H_ij x_j|.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

K, N, RMAX, Q, MAXK, LMAX = 7, 200, 200.0, 10, 10, 5
GOLD = os.path.join(os.path.dirname(__file__), "golden", "order7_n200_counts.json")


@pytest.fixture(scope="module")
def handle(bs2e):
    t = bs2e.grids.explin_knots(K, N, RMAX)
    h = bs2e.Bs2e(t, K, Q, MAXK)
    h.slater()
    h.rk()
    h.one_body(2, LMAX + 1, 2, 10.0, 0.0, copy_out=False)  # eta = 0: no absorbing potential
    yield h
    h.close()


def _cf(bs2e, L, spin):
    return bs2e.configs(L, L % 2, LMAX, N, K, spin=spin)


def test_block_counts_match_oracle_golden(bs2e, handle):
    gold = json.load(open(GOLD))["blocks"]
    assert len(gold) == 8
    for b in gold:
        cf = _cf(bs2e, b["L"], b["spin"])
        assert cf.size == b["rows"]
        assert handle.block_count(cf, b["L"], True, b["spin"]) == (b["nnz_H"], b["nnz_S"])


@pytest.mark.parametrize("kk", [0, 3, 10])
def test_rk_store_symmetries_and_positivity(handle, kk):
    E = handle.rk_export(kk)
    W = 2 * K - 1
    assert E.shape == (N, N, W, W)
    a, b, u, v = np.meshgrid(np.arange(N), np.arange(N), np.arange(W) - (K - 1),
                             np.arange(W) - (K - 1), indexing="ij")
    c, d = a + u, b + v
    ok = (c >= 0) & (c < N) & (d >= 0) & (d < N)
    a, b, u, v, c, d = (x[ok] for x in (a, b, u, v, c, d))
    R = E[a, b, u + K - 1, v + K - 1]
    assert (R > 0).all()
    assert (E[~ok] == 0).all()
    for other in (E[c, b, -u + K - 1, v + K - 1],   # R[c,b,a,d]
                  E[a, d, u + K - 1, -v + K - 1],   # R[a,d,c,b]
                  E[b, a, v + K - 1, u + K - 1]):   # R[b,a,d,c]
        assert np.abs(other - R).max() <= 1e-13 * R.max()
        assert (np.abs(other - R) / R).max() <= 1e-12


def _device_block(torch, handle, cf, L, spin, full):
    dev = torch.device("cuda", 0)
    nH, nS = handle.block_count(cf, L, full, spin)
    n = cf.size
    H = dict(index_ptr=torch.empty(n + 1, dtype=torch.int64, device=dev),
             indices=torch.empty(nH, dtype=torch.int64, device=dev),
             data=torch.empty(nH, dtype=torch.complex128, device=dev))
    S = dict(index_ptr=torch.empty(n + 1, dtype=torch.int64, device=dev),
             indices=torch.empty(max(nS, 1), dtype=torch.int64, device=dev),
             data=torch.empty(max(nS, 1), dtype=torch.complex128, device=dev))
    handle.block_fill_into(cf, L, full, spin, {k: t.data_ptr() for k, t in H.items()},
                           {k: t.data_ptr() for k, t in S.items()}, on_device=True)
    del S
    return H, nH


def _mv(torch, handle, op, H, nnz, n, x, data=None):
    y = torch.empty(n, dtype=torch.complex128, device=x.device)
    d = H["data"] if data is None else data
    # the inputs were made on torch's stream, the library runs on its own
    # (and synchronises it before returning)
    torch.cuda.synchronize()
    handle.csr_mv_device(op, n, n, nnz, H["index_ptr"].data_ptr(), H["indices"].data_ptr(),
                         d.data_ptr(), x.data_ptr(), y.data_ptr())
    return y


@pytest.mark.parametrize("L,spin", [(0, 0), (1, 1)])
def test_block_symmetric_without_cap(bs2e, handle, L, spin):
    torch = pytest.importorskip("torch")
    cf = _cf(bs2e, L, spin)
    n = cf.size
    gen = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn(n, dtype=torch.complex128, device="cuda", generator=gen)
    H, nH = _device_block(torch, handle, cf, L, spin, True)
    assert float(H["data"].imag.abs().max()) == 0.0  # real with eta = 0
    y = _mv(torch, handle, 0, H, nH, n, x)
    yt = _mv(torch, handle, 1, H, nH, n, x)
    scale = _mv(torch, handle, 0, H, nH, n, x.abs().to(torch.complex128),
                data=H["data"].abs().to(torch.complex128)).real
    del H
    torch.cuda.empty_cache()
    assert float(scale.min()) > 0.0  # every row holds entries
    assert float(((y - yt).abs() / scale).max()) <= 1e-12
    U, nU = _device_block(torch, handle, cf, L, spin, False)
    assert nU < nH
    ys = _mv(torch, handle, 2, U, nU, n, x)
    del U
    torch.cuda.empty_cache()
    assert float(((ys - y).abs() / scale).max()) <= 1e-12
