"""Known-answer tests that pin the oracle's binning restatement.

* core/unit_test/tstLinkedCellList.hpp:26-440: a 10^3 grid of unit cells,
  one particle per cell centre, created i-fastest so the binned order
  (i slowest, k fastest) reverses it; full and partial (250..750) ranges.
* core/unit_test/tstSort.hpp:60-200: reversed keys give a reversed
  permutation.
"""
import numpy as np
import pytest

NX = 10


def lcl_particles():
    pos = np.zeros((NX ** 3, 3))
    ids = np.zeros((NX ** 3, 3), np.int64)
    for k in range(NX):
        for j in range(NX):
            for i in range(NX):
                pid = i + j * NX + k * NX * NX
                ids[pid] = (i, j, k)
                pos[pid] = (i + 0.5, j + 0.5, k + 0.5)
    return pos, ids


@pytest.mark.parametrize("begin,end", [(0, 1000), (250, 750)])
def test_linked_cell_list(oracle, begin, end):
    pos, ids = lcl_particles()
    nb, counts, offsets, permutes = oracle.linked_cell_build(pos, begin, end, (0, 0, 0), (10, 10, 10), (1, 1, 1))
    assert tuple(nb) == (10, 10, 10)
    counts = counts.reshape(NX, NX, NX)
    offsets = offsets.reshape(NX, NX, NX)
    # permute the ids over [begin, end) (permute(lcl, aosoa), LinkedCellList.hpp:1130-1146)
    sorted_ids = ids.astype(np.float64).copy()
    oracle.permute(permutes, begin, end, sorted_ids)
    pid = 0
    for i in range(NX):
        for j in range(NX):
            for k in range(NX):
                orig = i + j * NX + k * NX * NX
                if begin <= orig < end:
                    assert tuple(sorted_ids[begin + pid].astype(int)) == (i, j, k)
                    assert counts[i, j, k] == 1
                    assert offsets[i, j, k] == pid
                    pid += 1
    n = 0
    for k in range(NX):
        for j in range(NX):
            for i in range(NX):
                if not (begin <= n < end):
                    assert tuple(sorted_ids[n].astype(int)) == (i, j, k)
                    assert counts[i, j, k] == 0
                n += 1


def test_bin_by_key_reversed(oracle):
    n = 1000
    keys = np.arange(n - 1, -1, -1, dtype=np.int32)
    counts, offsets, permutes = oracle.bin_by_key(keys, n)
    assert (counts == 1).all()
    assert (offsets == np.arange(n)).all()
    assert (permutes == np.arange(n - 1, -1, -1)).all()


def test_linked_cell_stable_within_bins(oracle):
    rng = np.random.default_rng(11)
    pos = rng.uniform(0, 4, size=(3000, 3))
    nb, counts, offsets, permutes = oracle.linked_cell_build(pos, 0, 3000, (0, 0, 0), (4, 4, 4), (1, 1, 1))
    cells = np.floor(pos).astype(np.int64)
    keys = (cells[:, 0] * 4 + cells[:, 1]) * 4 + cells[:, 2]
    assert (np.bincount(keys, minlength=64) == counts).all()
    assert (permutes.astype(np.int64) == np.argsort(keys, kind="stable")).all()
