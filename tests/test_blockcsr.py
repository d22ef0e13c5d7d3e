"""One CSR matrix from a block matrix: CS_from_block / CSR_from_block and
CSR_from_block_diag (src/tools/block_tools.f90:153-234, 289-348).

The oracle restates the reference's loop and is pinned against a dense
assembly on CPU; the GPU join (bs2e_csr_from_blocks) must equal it bit for
bit (pure data movement), including empty blocks, blocks of different
widths, and the combined H / dipole layout of symmetry blocks plus L+-1
coupling blocks.
"""
import numpy as np
import pytest

from cases import CASES, blocks, oracle_reference


def _rand_block(rng, n, m, density):
    if density == 0:
        return dict(shape=(n, m), nnz=0)
    ptr, idx, dat = [1], [], []
    for i in range(n):
        cols = np.flatnonzero(rng.random(m) < density)
        idx.extend(cols + 1)
        dat.extend(rng.standard_normal(cols.size) + 1j * rng.standard_normal(cols.size))
        ptr.append(len(idx) + 1)
    if not idx:
        return dict(shape=(n, m), nnz=0)
    return dict(shape=(n, m), nnz=len(idx), index_ptr=np.array(ptr, np.int64),
                indices=np.array(idx, np.int64), data=np.array(dat, np.complex128))


def _dense(A):
    D = np.zeros(A["shape"], dtype=np.complex128)
    if A["nnz"]:
        for i in range(A["shape"][0]):
            for e in range(A["index_ptr"][i] - 1, A["index_ptr"][i + 1] - 1):
                D[i, A["indices"][e] - 1] += A["data"][e]
    return D


def _grid(rng, rows, cols, dens):
    return {(i, j): _rand_block(rng, rows[i], cols[j], dens[i][j])
            for i in range(len(rows)) for j in range(len(cols))}


GRID = ([5, 0, 9, 3], [4, 7, 2], [[0.3, 0.0, 0.5], [0.2, 0.2, 0.2], [0.0, 0.4, 0.1],
                                  [0.6, 0.6, 0.0]])


def test_oracle_join_matches_dense(oracle):
    rng = np.random.default_rng(2)
    rows, cols, dens = GRID
    G = _grid(rng, rows, cols, dens)
    C = oracle.csr_from_blocks(G, len(rows), len(cols))
    want = np.block([[_dense(G[(i, j)]) for j in range(len(cols))] for i in range(len(rows))])
    np.testing.assert_array_equal(_dense(C), want)
    assert C["index_ptr"][-1] - 1 == C["nnz"]


@pytest.mark.gpu
def test_gpu_join_matches_oracle(bs2e, oracle):
    rng = np.random.default_rng(4)
    rows, cols, dens = GRID
    G = _grid(rng, rows, cols, dens)
    want = oracle.csr_from_blocks(G, len(rows), len(cols))
    c = CASES["ref60"]
    with bs2e.Bs2e(oracle_reference("ref60")["knots"], c["k"], c["q"], c["max_k"]) as h:
        got = h.csr_from_blocks(G, len(rows), len(cols))
    for key in ("index_ptr", "indices", "data"):
        np.testing.assert_array_equal(got[key], want[key])
    assert got["shape"] == want["shape"]


@pytest.mark.gpu
def test_gpu_join_symmetry_and_dipole_blocks(bs2e, oracle):
    """H_diag blocks of small2 (L=0,1,2 singlet) with the L+-1 dipole blocks
    (length gauge, q=0) in the off-diagonal positions: the combined matrix of
    the large configuration."""
    c = CASES["small2"]
    ref = oracle_reference("small2")
    bl = [b for b in blocks(bs2e, "small2") if b[3] == 0 and b[0] <= 2]
    with bs2e.Bs2e(ref["knots"], c["k"], c["q"], c["max_k"]) as h:
        h.slater()
        h.rk()
        h.set_one_body(ref["H1p"], ref["S"])
        h.radial_dipole(0)
        H = [h.block(cf, L, True, spin)[0] for (L, M, par, spin, cf) in bl]
        for Hb, (L, M, par, spin, cf) in zip(H, bl):
            Hb["shape"] = (cf.size, cf.size)
        G = {}
        for i, (L1, M1, p1, s1, cf1) in enumerate(bl):
            for j, (L2, M2, p2, s2, cf2) in enumerate(bl):
                if i == j:
                    G[(i, j)] = H[i]
                elif abs(L1 - L2) == 1:
                    D = h.dip_block(cf1, (L1, M1, p1), cf2, (L2, M2, p2), 0)
                    G[(i, j)] = D if D["nnz"] else dict(shape=D["shape"], nnz=0)
                else:
                    G[(i, j)] = dict(shape=(cf1.size, cf2.size), nnz=0)
        n = len(bl)
        got = h.csr_from_blocks(G, n, n)
        diag = h.csr_from_block_diag(H)
    want = oracle.csr_from_blocks(G, n, n)
    for key in ("index_ptr", "indices", "data"):
        np.testing.assert_array_equal(got[key], want[key])
    wd = oracle.csr_from_blocks({(i, j): (H[i] if i == j else dict(
        shape=(H[i]["shape"][0], H[j]["shape"][1]), nnz=0)) for i in range(n) for j in range(n)},
        n, n)
    for key in ("index_ptr", "indices", "data"):
        np.testing.assert_array_equal(diag[key], wd[key])


@pytest.mark.gpu
def test_gpu_join_errors(bs2e):
    c = CASES["ref60"]
    with bs2e.Bs2e(oracle_reference("ref60")["knots"], c["k"], c["q"], c["max_k"]) as h:
        bad = {(0, 0): dict(shape=(2, 2), nnz=2, index_ptr=np.array([1, 5, 3]),
                            indices=np.array([1, 2]), data=np.ones(2, np.complex128))}
        with pytest.raises(bs2e.Bs2eError, match="index_ptr"):
            h.csr_from_blocks(bad, 1, 1)
        wide = {(0, 0): dict(shape=(1, 2), nnz=1, index_ptr=np.array([1, 2]),
                             indices=np.array([3]), data=np.ones(1, np.complex128))}
        with pytest.raises(bs2e.Bs2eError, match="width"):
            h.csr_from_blocks(wide, 1, 1)
        empty = {(0, 0): dict(shape=(0, 3), nnz=0)}
        out = h.csr_from_blocks(empty, 1, 1)
        assert list(out["index_ptr"]) == [1]
