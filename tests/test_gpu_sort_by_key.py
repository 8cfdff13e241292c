"""GPU binByKey / sortByKey (cgx_bin_by_key_range), bit-exact against the
oracle: Kokkos::BinOp1D bins (nbin + 1 of them over the keys' [min, max]),
stable order inside a bin, and for sortByKey key order inside a bin.

* core/unit_test/tstSort.hpp:22-104 (sortByKey) and :105-200 (binByKey with
  num_data - 1 bins): 3,453 reversed keys; the permuted fields come out in
  ascending order and binByKey reports num_data bins of one key each.
* Random keys over narrow, negative and full int32 ranges, sub-ranges
  [begin, end), one bin, equal keys, a single key and an empty range.
* permute of int32 / int64 members (moved bit for bit with the rest).
"""
import numpy as np
import pytest
import torch

from cabana_gb300 import core as C

pytestmark = pytest.mark.gpu

NUM_DATA = 3453


def _reversed_fields():
    rev = np.arange(NUM_DATA - 1, -1, -1)
    v0 = torch.tensor(rev[:, None] + np.arange(3)[None, :], dtype=torch.float32, device="cuda")
    v1 = torch.tensor(rev, dtype=torch.float64, device="cuda")
    v2 = torch.tensor(rev[:, None, None] + np.arange(3)[None, :, None] + np.arange(2)[None, None, :],
                      dtype=torch.float64, device="cuda")
    keys = torch.tensor(rev, dtype=torch.int32, device="cuda")
    return keys, v0, v1, v2


def _check_sorted_fields(v0, v1, v2):
    p = np.arange(NUM_DATA)
    assert np.array_equal(v0.cpu().numpy(), (p[:, None] + np.arange(3)[None, :]).astype(np.float32))
    assert np.array_equal(v1.cpu().numpy(), p.astype(np.float64))
    assert np.array_equal(v2.cpu().numpy(), p[:, None, None] + np.arange(3)[None, :, None] + np.arange(2)[None, None, :])


def test_bin_by_key_reference_case(oracle):
    keys, v0, v1, v2 = _reversed_fields()
    bd = C.binByKey(keys, NUM_DATA - 1)
    assert bd.numBin() == NUM_DATA
    counts, offsets, permutes = oracle.bin_by_key_range(keys.cpu().numpy(), NUM_DATA - 1)
    assert np.array_equal(bd.counts.cpu().numpy(), counts)
    assert np.array_equal(bd.offsets.cpu().numpy().astype(np.uint64), offsets)
    assert np.array_equal(bd.permutes.cpu().numpy().astype(np.uint64), permutes)
    assert all(bd.binSize(p) == 1 and bd.binOffset(p) == p for p in (0, 1, 1726, NUM_DATA - 1))
    C.permute(bd, v0, v1, v2)
    _check_sorted_fields(v0, v1, v2)


def test_sort_by_key_reference_case(oracle):
    keys, v0, v1, v2 = _reversed_fields()
    bd = C.sortByKey(keys)
    assert np.array_equal(bd.permutes.cpu().numpy(), np.arange(NUM_DATA - 1, -1, -1))
    counts, offsets, permutes = oracle.bin_by_key_range(keys.cpu().numpy(), NUM_DATA // 2, sort_within_bins=True)
    assert np.array_equal(bd.counts.cpu().numpy(), counts)
    assert np.array_equal(bd.offsets.cpu().numpy().astype(np.uint64), offsets)
    C.permute(bd, v0, v1, v2)
    _check_sorted_fields(v0, v1, v2)


@pytest.mark.parametrize("by_key", [False, True])
@pytest.mark.parametrize("lo,hi,nbin,n", [(0, 40, 37, 50000), (-500, 700, 37, 50000), (-2**31, 2**31 - 1, 1000, 200000),
                                          (5, 6, 9, 3000), (7, 8, 0, 3000), (-3, -3, 12, 3000)])
def test_random_keys_bit_exact(oracle, by_key, lo, hi, nbin, n):
    rng = np.random.default_rng(abs(lo) % 997 + nbin + n)
    keys = rng.integers(lo, hi, size=n, endpoint=True).astype(np.int32)
    begin, end = n // 10, n - n // 7
    counts, offsets, permutes = oracle.bin_by_key_range(keys, nbin, begin, end, sort_within_bins=by_key)
    tk = torch.tensor(keys, device="cuda")
    # binByKey, or the sortByKey ordering with this nbin (sortByKey itself
    # uses nbin = (end - begin) // 2)
    bd = C._bin_range(tk, nbin, begin, end, True, None, None) if by_key else C.binByKey(tk, nbin, begin, end)
    assert np.array_equal(bd.counts.cpu().numpy(), counts)
    assert np.array_equal(bd.offsets.cpu().numpy().astype(np.uint64), offsets)
    assert np.array_equal(bd.permutes.cpu().numpy().astype(np.uint64), permutes)


def test_sort_by_key_random_sorts(oracle):
    rng = np.random.default_rng(8)
    keys = rng.integers(-10**6, 10**6, size=100000).astype(np.int32)
    bd = C.sortByKey(torch.tensor(keys, device="cuda"))
    perm = bd.permutes.cpu().numpy()
    assert np.array_equal(perm, np.argsort(keys, kind="stable"))
    counts, offsets, permutes = oracle.bin_by_key_range(keys, keys.shape[0] // 2, sort_within_bins=True)
    assert np.array_equal(bd.counts.cpu().numpy(), counts)
    assert np.array_equal(perm.astype(np.uint64), permutes)


def test_single_key_and_empty_range(oracle):
    one = torch.tensor([42], dtype=torch.int32, device="cuda")
    bd = C.binByKey(one, 5)
    assert bd.numBin() == 6 and bd.binSize(0) == 1 and bd.permutation(0) == 0
    bd = C.sortByKey(one)  # nbin = 0: one bin
    assert bd.numBin() == 1 and bd.binSize(0) == 1 and bd.permutation(0) == 0
    keys = torch.arange(10, dtype=torch.int32, device="cuda")
    bd = C.binByKey(keys, 4, 6, 6)
    assert bd.numBin() == 5 and int(bd.counts.sum()) == 0 and int(bd.offsets.abs().sum()) == 0


def test_permute_moves_integer_members_bit_for_bit():
    """The reference permutes whole AoSoAs, int members included
    (tstSort.hpp's int member): int32 and int64 fields move bit for bit,
    including patterns that read as NaNs when taken as floats."""
    rng = np.random.default_rng(21)
    n = 5000
    keys = rng.integers(0, 300, size=n).astype(np.int32)
    ids32 = rng.integers(-2**31, 2**31 - 1, size=(n, 2), endpoint=True).astype(np.int32)
    ids32[200:204, 0] = [0x7FC00001, -1, 0x7F800001, -0x7FFFFFFF]  # inside the permuted range
    ids64 = rng.integers(-2**63, 2**63 - 1, size=n, endpoint=True, dtype=np.int64)
    ids64[200:203] = [0x7FF0000000000001, -1, 0x7FF8000000000123]
    t32 = torch.tensor(ids32, device="cuda")
    t64 = torch.tensor(ids64, device="cuda")
    bd = C.binByKey(torch.tensor(keys, device="cuda"), 299, 100, 4900)
    C.permute(bd, t32, t64)
    perm = bd.permutes.cpu().numpy()
    r32, r64 = ids32.copy(), ids64.copy()
    r32[100:4900] = ids32[perm]
    r64[100:4900] = ids64[perm]
    assert np.array_equal(t32.cpu().numpy(), r32)
    assert np.array_equal(t64.cpu().numpy(), r64)
