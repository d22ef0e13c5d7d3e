"""The gfortran unformatted writer against an independent reader.

H_diag.dat / S_diag.dat / D_q.dat are what the reference's downstream
programs load (block_diag_CS%load, block_CS%load), so the library's writer must
produce the record layout of CS_block_diag_store / CS_block_store
(src/tools/block_tools.f90:386-485) in gfortran's record format, including
records split into subrecords above 2 GiB (exercised here with a small
subrecord size)."""
import numpy as np
import pytest

from cases import CASES, blocks, oracle_reference
from fortran_records import read_block, read_block_diag, read_records


def _oracle_blocks(bs2e, oracle):
    c = CASES["small2"]
    ref = oracle_reference("small2")
    out = []
    for (L, M, par, spin, cf) in blocks(bs2e, "small2")[:4]:
        H, S = oracle.construct_block(cf, L, c["k"], c["n_b"], c["max_k"], ref["R"], ref["H1p"],
                                      ref["S"], True, spin)
        H["shape"] = S["shape"] = (cf.size, cf.size)
        out.append((H, S))
    return out


@pytest.mark.parametrize("max_sub", [0, 1000, 37])
def test_block_diag_roundtrip(bs2e, oracle, tmp_path, max_sub):
    bl = _oracle_blocks(bs2e, oracle)
    Hs = [h for h, s in bl]
    empty = dict(shape=(5, 5), nnz=0)
    Hs.insert(1, empty)  # an empty block writes only shape and nnz
    p = tmp_path / "H_diag.dat"
    bs2e.write_block_diag(str(p), Hs, max_subrecord=max_sub)
    got = read_block_diag(str(p))
    assert got["block_shape"] == (len(Hs), len(Hs))
    assert got["shape"] == tuple(np.sum([b["shape"] for b in Hs], axis=0))
    for want, have in zip(Hs, got["blocks"]):
        assert have["shape"] == tuple(want["shape"]) and have["nnz"] == want["nnz"]
        if want["nnz"]:
            np.testing.assert_array_equal(have["index_ptr"], want["index_ptr"])
            np.testing.assert_array_equal(have["indices"], want["indices"])
            np.testing.assert_array_equal(have["data"], want["data"])
    if max_sub:
        # the data records are longer than max_sub and must be split
        recs = read_records(str(p))
        assert max(len(r) for r in recs) > max_sub


def test_record_layout_bytes(bs2e, tmp_path):
    p = tmp_path / "tiny.dat"
    blk = dict(shape=(1, 1), nnz=1, index_ptr=np.array([1, 2]), indices=np.array([1]),
               data=np.array([2.5 - 1j]))
    bs2e.write_block_diag(str(p), [blk])
    raw = p.read_bytes()
    # 'CSR' record: marker 3, bytes, marker 3
    assert raw[:11] == b"\x03\x00\x00\x00CSR\x03\x00\x00\x00"
    recs = read_records(str(p))
    assert [len(r) for r in recs] == [3, 16, 16, 16, 8, 16, 8, 16]


def test_block_file_roundtrip(bs2e, tmp_path):
    rng = np.random.default_rng(5)
    blocks_ = {}
    sizes = [3, 4]
    for j in range(2):
        for i in range(2):
            nr, nc = sizes[i], sizes[j]
            if i == j:
                blocks_[(i, j)] = dict(shape=(nr, nc), nnz=0)
                continue
            dense = (rng.random((nr, nc)) < 0.5) * (rng.random((nr, nc)) + 1j)
            ptr = [1]
            idx, dat = [], []
            for r in range(nr):
                for cc in range(nc):
                    if dense[r, cc] != 0:
                        idx.append(cc + 1)
                        dat.append(dense[r, cc])
                ptr.append(len(idx) + 1)
            blocks_[(i, j)] = dict(shape=(nr, nc), nnz=len(idx), index_ptr=np.array(ptr),
                                   indices=np.array(idx), data=np.array(dat, dtype=complex))
    p = tmp_path / "D_0.dat"
    bs2e.write_block(str(p), blocks_, 2, 2, max_subrecord=24)
    got = read_block(str(p))
    assert got["block_shape"] == (2, 2) and got["shape"] == (7, 7)
    for key, want in blocks_.items():
        have = got["blocks"][key]
        assert have["nnz"] == want["nnz"]
        if want["nnz"]:
            np.testing.assert_array_equal(have["indices"], want["indices"])
            np.testing.assert_array_equal(have["data"], want["data"])
