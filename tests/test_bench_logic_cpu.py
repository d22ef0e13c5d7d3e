"""Host-side logic of the bench's large job, without a GPU: the cut of the
job's units into chunks of nearly equal CSR bytes, the word views a digest
consumer reads out of a staging area, and the repeat check of the chunk
sums."""
import sys

import pytest
import torch

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _units(sizes):
    return [dict(bytes=int(b)) for b in sizes]


@pytest.mark.parametrize("n", [1, 3, 16])
def test_chunks_keep_unit_order_and_balance(n):
    sizes = [5, 1, 9, 2, 2, 7, 3, 8, 1, 6, 4, 4, 2, 9, 1, 3] * 3
    units = _units(sizes)
    chunks = bench.LargeJob._chunks(units, n)
    assert len(chunks) == n
    flat = [u for c in chunks for u in c]
    assert [id(u) for u in flat] == [id(u) for u in units]  # order kept, each once
    total = sum(sizes)
    acc = 0
    for i, c in enumerate(chunks[:-1]):
        acc += sum(u["bytes"] for u in c)
        # every cut is the first unit boundary at or past i+1 n-ths of the bytes
        assert acc >= total * (i + 1) / n
        assert acc - c[-1]["bytes"] < total * (i + 1) / n


def test_chunks_pad_with_empty_chunks():
    chunks = bench.LargeJob._chunks(_units([10, 10]), 5)
    assert len(chunks) == 5 and sum(len(c) for c in chunks) == 2


class _Job:
    """Just the attributes the word view and the repeat check use."""

    def __init__(self, areas=None, digests=None):
        self.torch = torch
        self.areas = areas or []
        self.digests = digests or {}


def test_words_view_an_area_by_address():
    area = torch.arange(64, dtype=torch.float64)
    job = _Job(areas=[area])
    w = bench.LargeJob._words(job, 0, area.data_ptr() + 8 * 5, 4)
    assert w.dtype == torch.int64 and w.numel() == 4
    assert torch.equal(w, area[5:9].view(torch.int64))
    with pytest.raises(AssertionError):  # past the end of the area
        bench.LargeJob._words(job, 0, area.data_ptr() + 8 * 62, 4)
    with pytest.raises(AssertionError):  # not on an 8-byte boundary
        bench.LargeJob._words(job, 0, area.data_ptr() + 4, 1)


def test_repeat_check_compares_bits():
    one = lambda v, dt: torch.tensor(v, dtype=dt)
    job = _Job(digests={0: [one(7, torch.int64), one(7, torch.int64)],
                        1: [one(3, torch.int64)],
                        2: [one(1 + 2j, torch.complex128), one(1 + 2j, torch.complex128)]})
    assert bench.LargeJob.digest_repeats(job) == (2, True)
    job.digests[2].append(one(1 + 2.0000000000000004j, torch.complex128))
    assert bench.LargeJob.digest_repeats(job) == (2, False)
    job.digests[2][-1] = one(complex(1, 2), torch.complex128)
    # -0.0 and +0.0 compare equal as numbers but not as bits
    job.digests[3] = [one(complex(0.0, 0.0), torch.complex128),
                      one(complex(-0.0, 0.0), torch.complex128)]
    assert bench.LargeJob.digest_repeats(job) == (3, False)
