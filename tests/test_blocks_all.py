"""bs2e_blocks_count_all / bs2e_blocks_fill_all: every symmetry block of a
basis in one call (the loop of main_basis_setup.f90:105-116 over bas%syms).
They must give exactly what the single-block calls give, block by block, into
host or device arrays, and name the failing block in the error message."""
import numpy as np
import pytest

from cases import CASES, blocks, oracle_reference

pytestmark = pytest.mark.gpu


def _handle(bs2e, case="small2"):
    c = CASES[case]
    ref = oracle_reference(case)
    h = bs2e.Bs2e(ref["knots"], c["k"], c["q"], c["max_k"])
    h.slater()
    h.rk()
    h.set_one_body(ref["H1p"], ref["S"])
    return h


def _same(a, b):
    for x in ("index_ptr", "indices", "data"):
        np.testing.assert_array_equal(a[x], b[x])


@pytest.mark.parametrize("full", [True, False])
def test_all_blocks_equal_single_block_calls(bs2e, oracle, full):
    c = CASES["small2"]
    bl = blocks(bs2e, "small2")
    spec = [(cf, L, spin) for (L, M, par, spin, cf) in bl]
    with _handle(bs2e) as h:
        nH, nS = h.blocks_count_all(spec, full)
        for (cf, L, spin), a, b in zip(spec, nH, nS):
            assert (a, b) == oracle.count_nnz(cf, L, c["k"], c["max_k"], full, spin)
        got = h.blocks_all(spec, full)
        for (cf, L, spin), (H, S) in zip(spec, got):
            Hr, Sr = h.block(cf, L, full, spin)
            _same(H, Hr)
            _same(S, Sr)


def test_all_blocks_into_device_arrays(bs2e):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    spec = [(cf, L, spin) for (L, M, par, spin, cf) in blocks(bs2e, "small2")]
    with _handle(bs2e) as h:
        nH, nS = h.blocks_count_all(spec, True)
        mk = lambda n, dt: torch.empty(max(int(n), 1), dtype=dt, device=dev)
        Ht, St = [], []
        for (cf, L, spin), a, b in zip(spec, nH, nS):
            n = cf.size
            Ht.append(dict(index_ptr=mk(n + 1, torch.int64), indices=mk(a, torch.int64),
                           data=mk(a, torch.complex128)))
            St.append(dict(index_ptr=mk(n + 1, torch.int64), indices=mk(b, torch.int64),
                           data=mk(b, torch.complex128)))
        addr = lambda D: {x: t.data_ptr() for x, t in D.items()}
        h.blocks_fill_all_into(spec, True, [addr(d) for d in Ht], [addr(d) for d in St],
                               on_device=True)
        host = h.blocks_all(spec, True)
    for (H, S), Hd, Sd in zip(host, Ht, St):
        for x in ("index_ptr", "indices", "data"):
            np.testing.assert_array_equal(Hd[x].cpu().numpy()[:H[x].size], H[x])
            np.testing.assert_array_equal(Sd[x].cpu().numpy()[:S[x].size], S[x])


def test_failing_block_is_named_and_empty_call_is_fine(bs2e):
    spec = [(cf, L, spin) for (L, M, par, spin, cf) in blocks(bs2e, "small2")]
    with _handle(bs2e) as h:
        assert [len(x) for x in h.blocks_count_all([], True)] == [0, 0]
        assert h.blocks_all([], True) == []
        cf, L, spin = spec[2]
        bad = cf[::-1].copy()  # not in basis order
        with pytest.raises(bs2e.Bs2eError, match="block 1:"):
            h.blocks_count_all([spec[0], (bad, L, spin), spec[1]], True)
        # the handle stays usable
        nH, nS = h.blocks_count_all(spec[:2], True)
        assert nH[0] > 0
