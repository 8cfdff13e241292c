"""Host logic of the Python LinkedCellList mirror on the CPU.

The two build entry points of libcgx run on the GPU; here a stand-in fills
their outputs from the oracle (the GPU results are bit-exact with it, see
tests/test_gpu_binning.py), so the mirror's own bookkeeping runs without a
GPU: 2D / 3D dispatch, rebuild, ranges, ijkBinIndex, and the per-particle
bins of LinkedCellList::storeParticleBins before and after the list is
marked sorted (Cabana_LinkedCellList.hpp:778-835, :1130-1146).
"""
import ctypes
import types

import numpy as np
import pytest
import torch

from cabana_gb300 import _lib as L
from cabana_gb300 import core as C


class _FakeLib:
    """Forwards host-only calls to libcgx and builds the lists with the oracle."""

    def __init__(self, oracle, positions):
        self.oracle = oracle
        self.positions = positions
        self.real = L.lib()
        self.builds = []

    def __getattr__(self, name):
        return getattr(self.real, name)

    def _fill(self, nd, begin, end, mn, mx, dl, counts_p, offsets_p, permutes_p):
        grid = [list(a)[:nd] for a in (mn, mx, dl)]
        _, counts, offsets, permutes = self.oracle.linked_cell_build(self.positions, begin, end, *grid)
        for arr, ptr in ((counts, counts_p), (offsets, offsets_p), (permutes, permutes_p)):
            ctypes.memmove(ptr.value, arr.ctypes.data, arr.nbytes)
        self.builds.append((nd, begin, end))
        return 0

    def cgx_linked_cell_build(self, h, desc, begin, end, mn, mx, dl, counts_p, offsets_p, permutes_p, stream):
        return self._fill(3, begin, end, mn, mx, dl, counts_p, offsets_p, permutes_p)

    def cgx_linked_cell_build_2d(self, h, desc, begin, end, mn, mx, dl, counts_p, offsets_p, permutes_p, stream):
        return self._fill(2, begin, end, mn, mx, dl, counts_p, offsets_p, permutes_p)


@pytest.fixture
def fake(monkeypatch, oracle):
    def install(positions):
        lib = _FakeLib(oracle, positions)
        monkeypatch.setattr(L, "lib", lambda: lib)
        monkeypatch.setattr(L, "default_handle", lambda: types.SimpleNamespace(ptr=None))
        monkeypatch.setattr(C, "field_descriptor", lambda f: L.CgxField())
        monkeypatch.setattr(C, "_stream", lambda s: ctypes.c_void_p(0))
        return lib
    return install


def _expected_bins(oracle, pos, begin, end, grid):
    nb, counts, offsets, permutes = oracle.linked_cell_build(pos, begin, end, *grid)
    in_order = np.repeat(np.arange(counts.shape[0]), counts)
    unsorted = np.empty(end - begin, np.int64)
    unsorted[permutes.astype(np.int64) - begin] = in_order
    return nb, in_order, unsorted


@pytest.mark.parametrize("nd", [3, 2])
def test_particle_bins_before_and_after_sorting(fake, oracle, nd):
    rng = np.random.default_rng(5 + nd)
    lo, hi, delta = (0.0, -1.0, 2.0)[:nd], (3.0, 2.0, 4.5)[:nd], (0.5, 0.75, 0.5)[:nd]
    pos = rng.uniform(lo, hi, size=(900, nd))
    lib = fake(pos)
    lcl = C.createLinkedCellList(torch.tensor(pos), delta, lo, hi, 100, 800)
    assert lib.builds == [(nd, 100, 800)]
    nb, in_order, unsorted = _expected_bins(oracle, pos, 100, 800, (lo, hi, delta))
    assert tuple(lcl.numBin(d) for d in range(nd)) == tuple(nb)
    assert lcl.numParticles() == 700 and (lcl.getParticleBegin(), lcl.getParticleEnd()) == (100, 800)
    assert (lcl.rangeBegin(), lcl.rangeEnd()) == (100, 800)
    assert not lcl.sorted()
    assert np.array_equal(lcl.getParticleBins().numpy(), unsorted)
    for p in (100, 431, 799):
        b = lcl.getParticleBin(p)
        assert b == unsorted[p - 100]
        assert lcl.cardinalBinIndex(*lcl.ijkBinIndex(b)) == b
    with pytest.raises(IndexError):
        lcl.getParticleBin(800)
    # permute(lcl, ...) marks the list sorted; the bins follow bin order
    C.permute(lcl)
    assert lcl.sorted()
    assert np.array_equal(lcl.getParticleBins().numpy(), in_order)
    lcl.update(False)
    assert np.array_equal(lcl.storeParticleBins().numpy(), unsorted)
    # rebuild over all particles with the same grid: not sorted again
    lcl.update(True)
    lcl.build(torch.tensor(pos))
    assert lib.builds[-1] == (nd, 0, 900) and not lcl.sorted()
    _, _, unsorted_all = _expected_bins(oracle, pos, 0, 900, (lo, hi, delta))
    assert np.array_equal(lcl.getParticleBins().numpy(), unsorted_all)
    with pytest.raises(ValueError):
        lcl.build(torch.tensor(pos), 10, 901)


def test_ijk_bin_index_round_trip(fake, oracle):
    pos = np.full((4, 3), 0.5)
    fake(pos)
    lcl = C.createLinkedCellList(torch.tensor(pos), (1.0, 0.5, 0.25), (0.0, 0.0, 0.0), (4.0, 3.0, 2.0))
    assert tuple(lcl.numBin(d) for d in range(3)) == (4, 6, 8)
    assert lcl.ijkBinIndex(0) == (0, 0, 0)
    assert lcl.ijkBinIndex(1) == (0, 0, 1)  # k fastest
    assert lcl.ijkBinIndex(8) == (0, 1, 0)
    assert lcl.ijkBinIndex(4 * 6 * 8 - 1) == (3, 5, 7)
    for c in range(0, 4 * 6 * 8, 7):
        assert lcl.cardinalBinIndex(lcl.ijkBinIndex(c)) == c


class _FakeSortLib(_FakeLib):
    """cgx_bin_by_key_range from the oracle, reading the keys the mirror passes."""

    def cgx_bin_by_key_range(self, h, keys_p, begin, end, nbin, sort_within, counts_p, offsets_p, permutes_p,
                             stream):
        n = end
        keys = np.ctypeslib.as_array(ctypes.cast(keys_p.value, ctypes.POINTER(ctypes.c_int32)), shape=(n,)).copy()
        self.keys_seen = keys
        counts, offsets, permutes = self.oracle.bin_by_key_range(keys, nbin, begin, end, bool(sort_within))
        for arr, ptr in ((counts, counts_p), (offsets, offsets_p), (permutes, permutes_p)):
            ctypes.memmove(ptr.value, arr.ctypes.data, arr.nbytes)
        return 0


def test_sort_and_bin_by_key_slice(monkeypatch, oracle):
    """tstSort.hpp:202-420 (sortByKey / binByKey of a slice): keys taken from
    an int member of an AoSoA (vector length 8, two int members per SoA)."""
    lib = _FakeSortLib(oracle, None)
    monkeypatch.setattr(L, "lib", lambda: lib)
    monkeypatch.setattr(L, "default_handle", lambda: types.SimpleNamespace(ptr=None))
    monkeypatch.setattr(C, "_stream", lambda s: ctypes.c_void_p(0))
    n, vl = 100, 8
    nsoa = (n + vl - 1) // vl
    storage = torch.full((nsoa * 2 * vl,), -7, dtype=torch.int32)
    rev = torch.arange(n - 1, -1, -1, dtype=torch.int32)
    i = torch.arange(n)
    storage[(i // vl) * 2 * vl + vl + i % vl] = rev  # member 1: keys(p) = reverse index
    keys = C.Slice(storage, vl, vl, 2 * vl, 1, n)
    bd = C.sortByKey(keys)
    assert np.array_equal(lib.keys_seen, rev.numpy())
    assert np.array_equal(bd.permutes.numpy(), np.arange(n - 1, -1, -1))
    bd = C.binByKey(keys, n - 1)
    assert bd.numBin() == n and (bd.counts.numpy() == 1).all()
    assert np.array_equal(bd.offsets.numpy(), np.arange(n))
    with pytest.raises(ValueError):
        C.binByKey(C.Slice(storage, 0, vl, 2 * vl, 2, n), 4)
    with pytest.raises(TypeError):
        C.binByKey(torch.zeros(5), 4)


def test_permute_descriptor_of_integer_members():
    """Integer members travel as the float type of their size (permute moves
    bits), for tensors and for Slices of an AoSoA's int storage."""
    storage = torch.zeros(64, dtype=torch.int32)
    d = C._move_descriptor(C.Slice(storage, 8, 8, 16, 1, 30))
    assert d.dtype == L.CGX_F32 and d.data == storage.data_ptr() + 8 * 4
    assert (d.vector_length, d.soa_stride, d.comp_stride) == (8, 16, 8)
    d = C._move_descriptor(C.Slice(torch.zeros(32, dtype=torch.int64), 0, 4, 8, 2, 12))
    assert d.dtype == L.CGX_F64
    with pytest.raises(TypeError):
        C._move_descriptor(C.Slice(torch.zeros(32, dtype=torch.int16), 0, 4, 8, 1, 12))
