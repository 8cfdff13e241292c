"""GPU binning parity, bit-exact against the oracle: LinkedCellList counts,
offsets and permutation (stable in-bin order), binning by bin number, permute, and the
tile-major ordering used by the tiled kernels."""
import numpy as np
import pytest
import torch

from cabana_gb300 import core as C
from cabana_gb300 import grid as G
from cabana_gb300 import mesh as M
from tests.helpers import clumped_points, domain, oracle_mesh

pytestmark = pytest.mark.gpu

NX = 10


def lcl_particles():
    pos = np.zeros((NX ** 3, 3))
    ids = np.zeros((NX ** 3, 3))
    for k in range(NX):
        for j in range(NX):
            for i in range(NX):
                pid = i + j * NX + k * NX * NX
                ids[pid] = (i, j, k)
                pos[pid] = (i + 0.5, j + 0.5, k + 0.5)
    return pos, ids


@pytest.mark.parametrize("begin,end", [(0, 1000), (250, 750)])
def test_linked_cell_list_reference_case(oracle, begin, end):
    """tstLinkedCellList.hpp:26-440 on the GPU, AoSoA-style permute of ids."""
    pos, ids = lcl_particles()
    tpos = torch.tensor(pos, device="cuda")
    tids = torch.tensor(ids, device="cuda")
    lcl = C.createLinkedCellList(tpos, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), (10.0, 10.0, 10.0), begin, end)
    assert lcl.totalBins() == 1000 and all(lcl.numBin(d) == 10 for d in range(3))
    nb, counts, offsets, permutes = oracle.linked_cell_build(pos, begin, end, (0, 0, 0), (10, 10, 10), (1, 1, 1))
    bd = lcl.binningData()
    assert np.array_equal(bd.counts.cpu().numpy(), counts)
    assert np.array_equal(bd.offsets.cpu().numpy().astype(np.uint64), offsets)
    assert np.array_equal(bd.permutes.cpu().numpy().astype(np.uint64), permutes)
    C.permute(lcl, tpos, tids)
    sorted_ids = ids.copy()
    oracle.permute(permutes, begin, end, sorted_ids)
    assert np.array_equal(tids.cpu().numpy(), sorted_ids)
    pid = 0
    for i in range(NX):
        for j in range(NX):
            for k in range(NX):
                orig = i + j * NX + k * NX * NX
                if begin <= orig < end:
                    assert tuple(sorted_ids[begin + pid].astype(int)) == (i, j, k)
                    assert lcl.binSize(i, j, k) == 1
                    assert lcl.binOffset(i, j, k) == pid
                    pid += 1


@pytest.mark.parametrize("begin,end", [(0, 100), (25, 75)])
def test_linked_cell_list_2d_reference_case(oracle, begin, end):
    """tstLinkedCellList.hpp's 2D case (LCLTestData<2>, checkLinkedCell
    :366-440) on the GPU: 10^2 unit cells, one particle per cell centre."""
    pos = np.array([(i + 0.5, j + 0.5) for j in range(NX) for i in range(NX)])
    ids = np.array([(i, j) for j in range(NX) for i in range(NX)], np.float64)
    tpos = torch.tensor(pos, device="cuda")
    tids = torch.tensor(ids, device="cuda")
    lcl = C.createLinkedCellList(tpos, (1.0, 1.0), (0.0, 0.0), (10.0, 10.0), begin, end)
    assert lcl.totalBins() == 100 and lcl.numBin(0) == 10 and lcl.numBin(1) == 10
    nb, counts, offsets, permutes = oracle.linked_cell_build(pos, begin, end, (0, 0), (10, 10), (1, 1))
    bd = lcl.binningData()
    assert np.array_equal(bd.counts.cpu().numpy(), counts)
    assert np.array_equal(bd.offsets.cpu().numpy().astype(np.uint64), offsets)
    assert np.array_equal(bd.permutes.cpu().numpy().astype(np.uint64), permutes)
    C.permute(lcl, tpos, tids)
    sorted_ids = ids.copy()
    oracle.permute(permutes, begin, end, sorted_ids)
    assert np.array_equal(tids.cpu().numpy(), sorted_ids)
    pid = 0
    for i in range(NX):
        for j in range(NX):
            if begin <= i + j * NX < end:
                assert tuple(sorted_ids[begin + pid].astype(int)) == (i, j)
                assert lcl.binSize(i, j) == 1 and lcl.binSize((i, j)) == 1
                assert lcl.binOffset(i, j) == pid
                pid += 1


@pytest.mark.parametrize("n,clumps", [(1, 0), (5000, 0), (200000, 2)])
def test_linked_cell_2d_random_bit_exact(oracle, n, clumps):
    rng = np.random.default_rng(70 + n)
    lo, hi = (0.0, -1.0), (6.3, 5.0)
    if clumps:
        centres = rng.uniform(lo, hi, size=(clumps, 2))
        pos = centres[rng.integers(0, clumps, n)] + rng.normal(0.0, 0.05, size=(n, 2))
        pos = np.clip(pos, lo, np.nextafter(np.array(hi), -np.inf))
    else:
        pos = rng.uniform(lo, hi, size=(n, 2))
    delta = (0.37, 0.5)
    nb, counts, offsets, permutes = oracle.linked_cell_build(pos, 0, n, lo, hi, delta)
    lcl = C.createLinkedCellList(torch.tensor(pos, device="cuda"), delta, lo, hi)
    assert (lcl.numBin(0), lcl.numBin(1)) == tuple(nb)
    bd = lcl.binningData()
    assert np.array_equal(bd.counts.cpu().numpy(), counts)
    assert np.array_equal(bd.offsets.cpu().numpy().astype(np.uint64), offsets)
    assert np.array_equal(bd.permutes.cpu().numpy().astype(np.uint64), permutes)


@pytest.mark.parametrize("n,clumps", [(1, 0), (5000, 0), (200000, 2), (300000, 1)])
def test_linked_cell_random_bit_exact(oracle, n, clumps):
    rng = np.random.default_rng(n)
    lo, hi = (0.0, -1.0, 2.0), (6.3, 5.0, 9.1)
    if clumps:
        pos = clumped_points(rng, n, lo, hi, clumps, 0.05)  # thousands per bin
    else:
        pos = rng.uniform(lo, hi, size=(n, 3))
    delta = (0.37, 0.5, 0.29)
    nb, counts, offsets, permutes = oracle.linked_cell_build(pos, 0, n, lo, hi, delta)
    lcl = C.createLinkedCellList(torch.tensor(pos, device="cuda"), delta, lo, hi)
    assert tuple(lcl.numBin(d) for d in range(3)) == tuple(nb)
    bd = lcl.binningData()
    assert np.array_equal(bd.counts.cpu().numpy(), counts)
    assert np.array_equal(bd.offsets.cpu().numpy().astype(np.uint64), offsets)
    assert np.array_equal(bd.permutes.cpu().numpy().astype(np.uint64), permutes)


def test_points_on_upper_boundary_go_to_last_bin(oracle):
    pos = np.array([[10.0, 10.0, 10.0], [0.0, 0.0, 0.0], [9.999, 10.0, 0.5]])
    nb, counts, offsets, permutes = oracle.linked_cell_build(pos, 0, 3, (0, 0, 0), (10, 10, 10), (1, 1, 1))
    lcl = C.createLinkedCellList(torch.tensor(pos, device="cuda"), (1, 1, 1), (0, 0, 0), (10, 10, 10))
    assert np.array_equal(lcl.binningData().counts.cpu().numpy(), counts)
    assert np.array_equal(lcl.binningData().permutes.cpu().numpy().astype(np.uint64), permutes)


def test_bin_by_index(oracle):
    """Binning by bin number (cgx_bin_by_key): reversed keys give the reversed
    permutation; plus a random key set with many duplicates (stable order)."""
    n = 3000
    keys = np.arange(n - 1, -1, -1, dtype=np.int32)
    bd = C.binByIndex(torch.tensor(keys, device="cuda"), n)
    assert np.array_equal(bd.permutes.cpu().numpy(), np.arange(n - 1, -1, -1))
    rng = np.random.default_rng(2)
    keys = rng.integers(0, 37, size=50000).astype(np.int32)
    counts, offsets, permutes = oracle.bin_by_key(keys, 37, 1000, 40000)
    bd = C.binByIndex(torch.tensor(keys, device="cuda"), 37, 1000, 40000)
    assert np.array_equal(bd.counts.cpu().numpy(), counts)
    assert np.array_equal(bd.offsets.cpu().numpy().astype(np.uint64), offsets)
    assert np.array_equal(bd.permutes.cpu().numpy().astype(np.uint64), permutes)


def test_permute_fields_f32_f64(oracle):
    rng = np.random.default_rng(4)
    n = 10000
    a = rng.normal(size=(n, 9))
    b = rng.normal(size=(n,)).astype(np.float32)
    ta = torch.tensor(a, device="cuda").reshape(n, 3, 3)
    tb = torch.tensor(b, device="cuda")
    pr = (100 + rng.permutation(8900)).astype(np.uint64)  # permutation of [100, 9000)
    bd = C.BinningData(100, 9000, torch.empty(0), torch.empty(0), torch.tensor(pr.astype(np.int64), device="cuda"))
    C.permute(bd, ta, tb)
    ra = a.copy()
    oracle.permute(pr, 100, 9000, ra)
    rb = b.astype(np.float64).copy().reshape(n, 1)
    oracle.permute(pr, 100, 9000, rb)
    assert np.array_equal(ta.cpu().numpy().reshape(n, 9), ra)
    assert np.array_equal(tb.cpu().numpy().astype(np.float64), rb[:, 0])


@pytest.mark.parametrize("order", [1, 2, 3])
def test_tile_sort_matches_stable_key_sort(oracle, order):
    lg, mp = M.simple_mesh((13, 9, 11), 0.5, (1.0, -2.0, 0.25), 2)
    rng = np.random.default_rng(order)
    n = 40000
    lo, hi = domain(mp)
    pts = clumped_points(rng, n, lo, hi, 2, 0.4)
    tile = (4, 4, 4)
    til = G.Tiling(mp, order, tile)
    perm = til.sort(torch.tensor(pts, device="cuda"), n).cpu().numpy().astype(np.uint64)
    # expected keys from the oracle's own stencil base
    om = oracle_mesh(oracle, mp)
    nt = tuple(til.struct.num_tiles)
    keys = np.zeros(n, np.uint64)
    counts = np.zeros(int(np.prod(nt)), np.int64)
    for p in range(n):
        s = oracle.evaluate_spline(om, order, pts[p])["s"][:, 0]
        t = [min(int(s[d]) // tile[d], nt[d] - 1) for d in range(3)]
        loc = [int(s[d]) - t[d] * tile[d] for d in range(3)]
        tid = (t[0] * nt[1] + t[1]) * nt[2] + t[2]
        keys[p] = tid * 64 + (loc[0] * 4 + loc[1]) * 4 + loc[2]
        counts[tid] += 1
    assert np.array_equal(perm, oracle.stable_sort_keys(keys))
    offs = til.offsets.cpu().numpy()
    assert offs[0] == 0 and np.array_equal(np.diff(offs), counts)
