"""CPU tests of the C-ABI library: it loads, exports every declared symbol,
and its host-side pieces (configuration lists, exact 3j/6j, grids) agree with
the oracle and the golden vectors.  No CUDA compute is called here."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

from cases import CASES
from conftest import ROOT, gpu_available

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "bs2e.h")).read()
    return sorted(set(re.findall(r"BS2E_API\s+[\w\s\*]+?\b(bs2e_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol(bs2e):
    names = declared_symbols()
    assert len(names) >= 20
    L = ctypes.CDLL(bs2e.LIB_PATH)
    for n in names:
        assert hasattr(L, n), n
    assert sorted(bs2e.EXPORTS) == names


def test_exact_wigner_vs_golden(bs2e):
    d = json.load(open(os.path.join(GOLD, "wigner.json")))
    for *a, v in d["three_j"]:
        assert abs(bs2e.three_j(*a) - v) <= 4.5e-16 * abs(v), a
    for *a, v in d["six_j"]:
        got = bs2e.six_j(*a)
        if v == 0.0:
            assert got == 0.0, a
        else:
            assert abs(got - v) <= 4.5e-16 * abs(v), a


def test_ang_k_LS_matches_oracle(bs2e, oracle):
    for la in range(0, 6):
        for lb in range(0, la + 1):
            for lc in range(0, 6):
                for ld in range(0, lc + 1):
                    for L in range(0, 4):
                        for k in range(0, 11):
                            a = bs2e.ang_k_LS(k, la, lb, lc, ld, L)
                            b = oracle.ang_k_LS(k, la, lb, lc, ld, L)
                            assert abs(a - b) <= 1e-14, (k, la, lb, lc, ld, L, a, b)


@pytest.mark.parametrize("spin", [0, 1])
def test_config_lists_match_oracle(bs2e, oracle, spin):
    for (L, par, lmax, nb, k, mnb, nal, l2m) in [(0, 0, 2, 60, 6, None, None, None),
                                                 (3, 1, 5, 40, 7, None, None, None),
                                                 (2, 0, 5, 40, 7, None, None, None),
                                                 (1, 0, 3, 24, 5, 15, 12, 1),
                                                 (2, 1, 4, 30, 6, 20, 25, 2)]:
        a = bs2e.configs(L, par, lmax, nb, k, mnb, nal, l2m, spin)
        b = oracle.count_configs(L, par, lmax, nb, k, mnb, nal, l2m, spin)
        assert a.size == b.size
        np.testing.assert_array_equal(a.view(np.int64), b.view(np.int64))


def test_explin_knots_sizes(bs2e):
    for (k, nb, rmax) in [(6, 60, 50.0), (7, 200, 200.0), (8, 400, 400.0), (9, 800, 800.0)]:
        t = bs2e.grids.explin_knots(k, nb, rmax)
        assert t.size - k - 2 == nb
        assert (np.diff(t) >= 0).all() and t[0] == 0 and t[-1] == rmax
        assert (t[:k] == 0).all() and (t[-k:] == rmax).all()
        n_iv = np.unique(t).size - 1
        assert n_iv == t.size - 2 * k + 1
    # order 6, 60 B-splines to r_max=50 has 57 breakpoint intervals
    assert np.unique(bs2e.grids.explin_knots(6, 60, 50.0)).size - 1 == 57


def test_generate_grid_restatement(bs2e):
    t = bs2e.grids.generate_grid(6, 3, 2, 0.5, 15.0)
    assert (t[:6] == 0).all() and (t[-6:] == t[-1]).all()
    assert t[-1] >= 15.0 and np.all(np.diff(t) >= 0)


def test_symmetry_order(bs2e):
    assert bs2e.basis.symmetries(3, True) == [(0, 0, 0), (1, 0, 1), (2, 0, 0), (3, 0, 1)]
    s = bs2e.basis.symmetries(2, False)
    assert len(s) == 9 and s[:4] == [(0, 0, 0), (1, 0, 0), (1, -1, 1), (1, 1, 1)]


def test_create_rejects_bad_input_without_gpu(bs2e):
    L = bs2e.lib()
    h = ctypes.c_void_p()
    bad = np.array([0.0, 1.0, 0.5, 2.0, 3.0, 3.0, 3.0, 3.0])  # decreasing knot
    assert L.bs2e_create(bs2e._ptr(bad), bad.size, 3, 4, 2, None, ctypes.byref(h)) == 1
    t = bs2e.grids.explin_knots(6, 30, 30.0)
    assert L.bs2e_create(bs2e._ptr(t), t.size, 1, 4, 2, None, ctypes.byref(h)) == 1  # k < 2
    assert L.bs2e_create(bs2e._ptr(t), t.size, 6, 0, 2, None, ctypes.byref(h)) == 1  # q < 1


def test_batched_block_calls_reject_bad_arguments_without_gpu(bs2e):
    L = bs2e.lib()
    z = np.zeros(1, dtype=np.int64)
    p = bs2e._ptr
    # no handle, and a negative block count: rejected before any device work
    assert L.bs2e_blocks_count_all(None, 1, None, p(z), p(z), p(z), 1, p(z), p(z)) == 1
    assert L.bs2e_blocks_fill_all(None, 0, None, None, None, None, 1, None, None, None, None,
                                  None, None, 0) == 1


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU failure path")
def test_compute_path_fails_loudly_without_gpu(bs2e):
    t = bs2e.grids.explin_knots(6, 30, 30.0)
    with pytest.raises(bs2e.Bs2eError) as e:
        bs2e.Bs2e(t, 6, 8, 4)
    assert e.value.status == 7  # BS2E_ERR_NODEV
