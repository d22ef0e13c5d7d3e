"""The plain-C caller (tests/capi_driver.c) against the oracle.

The driver includes include/bs2e.h and is compiled with gcc as strict C11
(warnings as errors) and linked against libbs2e.so, so the header meets a C
compiler and every entry point it calls resolves in the library.  On the GPU
it runs the shim's call sequence (create, slater, rk, one-body, count, fill,
rk_get, destroy) on the reference-sized case (order 6, N=60, k=0..4, singlet
L=0) and its CSR must equal the oracle's: pattern bit-exact, values within
1e-12 of their term scale.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from cases import CASES, blocks, knots, oracle_reference, assert_csr_close

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _driver():
    sys.path.insert(0, os.path.join(ROOT, "b-spline-two-e_gb300"))
    import build
    build.build()
    return build.build_driver()


def test_driver_compiles_against_header(bs2e):
    path = _driver()
    assert os.path.exists(path) and os.access(path, os.X_OK)


@pytest.mark.gpu
def test_driver_matches_oracle(bs2e, oracle, tmp_path):
    path = _driver()
    c = CASES["ref60"]
    ref = oracle_reference("ref60")
    t = knots(bs2e, "ref60")
    L, M, par, spin, cf = blocks(bs2e, "ref60")[0]
    n_l = c["lmax"] + 1
    hdr = np.array([c["k"], c["q"], c["max_k"], t.size, cf.size, L, 1, c["Z"], n_l, 2],
                   dtype=np.int64)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.array([10.0, 1e-3, 0.0]).tobytes())
        f.write(np.ascontiguousarray(t, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(cf).tobytes())
    r = subprocess.run([path, str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = open(out, "rb").read()
    off = 0

    def take(dt, n):
        nonlocal off
        a = np.frombuffer(raw, dtype=dt, count=n, offset=off)
        off += a.nbytes
        return a

    status, nH, nS, n_b, nnz4, nnz6 = take(np.int64, 6)
    assert status == 0 and n_b == c["n_b"]
    assert nnz4 == ref["prim"]["idx4"].shape[0] and nnz6 == ref["prim"]["idx6"].shape[0]
    n = cf.size
    H = dict(index_ptr=take(np.int64, n + 1), indices=take(np.int64, nH),
             data=take(np.complex128, nH))
    S = dict(index_ptr=take(np.int64, n + 1), indices=take(np.int64, nS),
             data=take(np.complex128, nS))
    rk = take(np.float64, 2 * (c["max_k"] + 1)).reshape(2, -1)
    assert off == len(raw)
    Hr, Sr = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"], ref["H1p"],
                                    ref["S"], True, spin)
    assert_csr_close(H, Hr)
    assert_csr_close(S, Sr, with_scale=False)
    want = oracle.rk_lookup(ref["R"], c["k"], [[1, 1, 1, 1], [2, 3, 1, 4]])
    np.testing.assert_allclose(rk, want, rtol=1e-12, atol=0)
