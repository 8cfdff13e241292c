"""Known-answer tests that pin the oracle's binning restatement.

* core/unit_test/tstLinkedCellList.hpp:26-440: a 10^3 grid of unit cells,
  one particle per cell centre, created i-fastest so the binned order
  (i slowest, k fastest) reverses it; full and partial (250..750) ranges.
  The 2D twin (LCLTestData<2>, :108-175, checkLinkedCell :366-440): a 10^2
  grid, 100 particles, full and partial (25..75) ranges.
* core/unit_test/tstSort.hpp:22-200: sortByKey and binByKey(keys,
  num_data - 1) of 3,453 reversed keys give the reversed permutation;
  binByKey has num_data bins (Kokkos::BinOp1D makes nbin + 1), one key each.
* binByKey / sortByKey on random keys against a numpy restatement of
  BinOp1D + a stable sort; binning by bin number (cgx_bin_by_key's contract)
  on reversed keys.
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


def lcl_particles_2d():
    pos = np.zeros((NX ** 2, 2))
    ids = np.zeros((NX ** 2, 2), np.int64)
    for j in range(NX):
        for i in range(NX):
            pid = i + j * NX
            ids[pid] = (i, j)
            pos[pid] = (i + 0.5, j + 0.5)
    return pos, ids


@pytest.mark.parametrize("begin,end", [(0, 100), (25, 75)])
def test_linked_cell_list_2d(oracle, begin, end):
    pos, ids = lcl_particles_2d()
    nb, counts, offsets, permutes = oracle.linked_cell_build(pos, begin, end, (0, 0), (10, 10), (1, 1))
    assert tuple(nb) == (10, 10)
    counts = counts.reshape(NX, NX)
    offsets = offsets.reshape(NX, NX)
    sorted_ids = ids.astype(np.float64).copy()
    oracle.permute(permutes, begin, end, sorted_ids)
    pid = 0
    for i in range(NX):
        for j in range(NX):
            orig = i + j * NX
            if begin <= orig < end:
                assert tuple(sorted_ids[begin + pid].astype(int)) == (i, j)
                assert counts[i, j] == 1
                assert offsets[i, j] == pid
                pid += 1
    n = 0
    for j in range(NX):
        for i in range(NX):
            if not (begin <= n < end):
                assert tuple(sorted_ids[n].astype(int)) == (i, j)
                assert counts[i, j] == 0
            n += 1


def test_linked_cell_2d_is_3d_with_one_z_cell(oracle):
    """2D keys i * ny + j equal the 3D keys of the same points with a single
    z cell, so the 2D build equals the 3D build with a constant z."""
    rng = np.random.default_rng(12)
    pos = rng.uniform((0.0, -1.0), (3.7, 2.0), size=(4000, 2))
    nb2, c2, o2, p2 = oracle.linked_cell_build(pos, 100, 3900, (0.0, -1.0), (3.7, 2.0), (0.31, 0.23))
    pos3 = np.concatenate([pos, np.full((4000, 1), 0.5)], axis=1)
    nb3, c3, o3, p3 = oracle.linked_cell_build(pos3, 100, 3900, (0.0, -1.0, 0.0), (3.7, 2.0, 1.0), (0.31, 0.23, 1.0))
    assert tuple(nb3) == tuple(nb2) + (1,)
    assert np.array_equal(c2, c3) and np.array_equal(o2, o3) and np.array_equal(p2, p3)


def test_bin_by_key_reference_case(oracle):
    num_data = 3453
    keys = np.arange(num_data - 1, -1, -1, dtype=np.int32)  # keys(p) = reverse index
    counts, offsets, permutes = oracle.bin_by_key_range(keys, num_data - 1)
    assert counts.shape[0] == num_data  # bin_data.numBin() == num_data
    assert (counts == 1).all()
    assert (offsets == np.arange(num_data)).all()
    assert (permutes == np.arange(num_data - 1, -1, -1)).all()


def test_sort_by_key_reference_case(oracle):
    num_data = 3453
    keys = np.arange(num_data - 1, -1, -1, dtype=np.int32)
    nbin = num_data // 2
    counts, offsets, permutes = oracle.bin_by_key_range(keys, nbin, sort_within_bins=True)
    assert (permutes == np.arange(num_data - 1, -1, -1)).all()
    # mul = 1726 / 3452: two keys per bin, the largest key alone in bin 1726
    assert counts.shape[0] == nbin + 1
    assert (counts[:-1] == 2).all() and counts[-1] == 1


def _bin_range_numpy(keys, nbin, begin, end, by_key):
    k = keys[begin:end].astype(np.int64)
    lo, hi = int(k.min()), int(k.max())
    rng = float(hi) - float(lo)
    mul = 1.0 if rng <= float(nbin) else float(nbin) / rng
    bins = (mul * (k.astype(np.float64) - float(lo))).astype(np.int64)
    counts = np.bincount(bins, minlength=nbin + 1)
    order = np.lexsort((k, bins)) if by_key else np.argsort(bins, kind="stable")
    return counts, np.concatenate([[0], np.cumsum(counts)[:-1]]), order + begin


@pytest.mark.parametrize("by_key", [False, True])
@pytest.mark.parametrize("lo,hi,nbin", [(0, 40, 37), (-500, 700, 37), (-2**31, 2**31 - 1, 1000), (5, 6, 9),
                                        (7, 8, 0)])
def test_bin_by_key_range_random(oracle, by_key, lo, hi, nbin):
    rng = np.random.default_rng(abs(lo) % 1000 + nbin)
    keys = rng.integers(lo, hi, size=6000, endpoint=True).astype(np.int32)
    begin, end = 300, 5700
    counts, offsets, permutes = oracle.bin_by_key_range(keys, nbin, begin, end, sort_within_bins=by_key)
    c2, o2, p2 = _bin_range_numpy(keys, nbin, begin, end, by_key)
    assert (counts == c2).all() and (offsets == o2).all()
    assert (permutes.astype(np.int64) == p2).all()


def test_bin_by_key_range_empty(oracle):
    counts, offsets, permutes = oracle.bin_by_key_range(np.zeros(10, np.int32), 4, 5, 5)
    assert counts.shape[0] == 5 and not counts.any() and not offsets.any() and permutes.shape[0] == 0


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
