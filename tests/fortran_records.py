"""Reader of gfortran unformatted sequential files (test infrastructure).

An independent implementation of gfortran's documented record format: every
logical record is one or more subrecords, each framed by 4-byte little-endian
markers; the leading marker is negative when more subrecords follow, the
trailing marker is negative when subrecords preceded.  Used to read back the
block CSR files the library writes (the layout of CS_block_diag_store and
CS_block_store, src/tools/block_tools.f90:386-485).
"""
import struct

import numpy as np


def read_records(path):
    out = []
    with open(path, "rb") as f:
        buf = f.read()
    pos = 0
    while pos < len(buf):
        data = bytearray()
        first = True
        while True:
            (lead,) = struct.unpack_from("<i", buf, pos)
            pos += 4
            n = abs(lead)
            data += buf[pos:pos + n]
            pos += n
            (trail,) = struct.unpack_from("<i", buf, pos)
            pos += 4
            assert abs(trail) == n, "marker mismatch"
            assert (trail > 0) == first, "trailing marker sign"
            first = False
            if lead > 0:
                break
        out.append(bytes(data))
    return out


def _block(recs, i):
    shape = tuple(np.frombuffer(recs[i], "<i8"))
    nnz = int(np.frombuffer(recs[i + 1], "<i8")[0])
    i += 2
    blk = dict(shape=shape, nnz=nnz)
    if nnz > 0:
        blk["index_ptr"] = np.frombuffer(recs[i], "<i8").copy()
        blk["indices"] = np.frombuffer(recs[i + 1], "<i8").copy()
        blk["data"] = np.frombuffer(recs[i + 2], "<c16").copy()
        i += 3
    return blk, i


def read_block_diag(path):
    """block_diag_CS%load (src/tools/block_tools.f90:487-520)."""
    recs = read_records(path)
    assert recs[0] == b"CSR"
    block_shape = tuple(np.frombuffer(recs[1], "<i8"))
    shape = tuple(np.frombuffer(recs[2], "<i8"))
    i, blocks = 3, []
    for _ in range(block_shape[0]):
        b, i = _block(recs, i)
        blocks.append(b)
    assert i == len(recs)
    return dict(block_shape=block_shape, shape=shape, blocks=blocks)


def read_block(path):
    """block_CS%load (src/tools/block_tools.f90:417-456); blocks[(i, j)]."""
    recs = read_records(path)
    assert recs[0] == b"CSR"
    block_shape = tuple(np.frombuffer(recs[1], "<i8"))
    shape = tuple(np.frombuffer(recs[2], "<i8"))
    i, blocks = 3, {}
    for j in range(block_shape[1]):
        for r in range(block_shape[0]):
            b, i = _block(recs, i)
            blocks[(r, j)] = b
    assert i == len(recs)
    return dict(block_shape=block_shape, shape=shape, blocks=blocks)
