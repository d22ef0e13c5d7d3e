"""The allocation-free R^k lookup against the allocating one.

bs2e_rk_get_batch_static serves callers that can't allocate device memory
when they look up R^k values -- for example a caller whose CSR blocks already
fill HBM, or one that can't let cudaFree wait for the whole device while other
streams work.  It stages keys and values in one static device array instead of
per-call buffers.  Two calls in a row with different keys must return exactly
what bs2e_rk_get_batch returns (both read the same store with the same
arithmetic), keys outside the basis or the band must give zeros in both, an
empty call must succeed, and a request beyond the array's capacity must be
refused with a clear error.  This file is collected last, after every other
test, and also passes on its own in a fresh process.
"""
import numpy as np
import pytest

from cases import CASES, knots

pytestmark = pytest.mark.gpu


def _keys(rng, N, k, n):
    a = rng.integers(1, N + 1, n)
    b = rng.integers(1, N + 1, n)
    c = np.clip(a + rng.integers(-(k - 1), k, n), 1, N)
    d = np.clip(b + rng.integers(-(k - 1), k, n), 1, N)
    return np.stack([a, b, c, d], axis=1).astype(np.int64)


def _outside(N, k):
    """Keys with an index outside 1..N or a pair outside the band |a-c| < k."""
    return np.array([[0, 1, 1, 1], [1, N + 1, 1, N], [N + 1, 1, N, 1], [1, 1, 1 + k, 1],
                     [2, 3, 2, 3 + k], [N, N, N - k, N]], dtype=np.int64)


@pytest.mark.parametrize("precision", [0, 1])
def test_static_lookup_matches_allocating_lookup(bs2e, precision):
    c = CASES["small2"]
    rng = np.random.default_rng(11)
    with bs2e.Bs2e(knots(bs2e, "small2"), c["k"], c["q"], c["max_k"], precision=precision) as h:
        h.slater()
        h.rk()
        assert h.rk_get_static(np.zeros((0, 4), dtype=np.int64)).shape == (0, h.K1)
        for n in (1500, 4096):  # two calls in a row; the second fills the scratch
            keys = _keys(rng, c["n_b"], c["k"], n)
            keys[:6] = _outside(c["n_b"], c["k"])
            want = h.rk_get(keys)
            got = h.rk_get_static(keys)
            assert (want[6:] > 0).all()
            assert (want[:6] == 0).all()
            np.testing.assert_array_equal(got, want)
        with pytest.raises(bs2e.Bs2eError) as e:
            h.rk_get_static(_keys(rng, c["n_b"], c["k"], 4097))
        assert e.value.status == 1 and "4096" in str(e.value)
