"""Cabana core binning API over torch CUDA tensors.

  LinkedCellList / createLinkedCellList  (core/src/Cabana_LinkedCellList.hpp:128-1146)
  BinningData                           (core/src/Cabana_Sort.hpp:37-136)
  binByKey / sortByKey                  (core/src/Cabana_Sort.hpp:217-235, :364-443)
  binByIndex (keys are bin numbers)     (the BinSort of core/src/Cabana_Sort.hpp:164-182)
  permute                               (core/src/Cabana_Sort.hpp:549-720)

All work runs in libcgx.so. Bins keep particles in ascending index order
(the reference's Serial-backend order), so results are deterministic.
"""
import ctypes
from dataclasses import dataclass

import torch

from . import _lib as L
from .grid import Slice, _stream, field_descriptor


@dataclass
class BinningData:
    begin: int
    end: int
    counts: torch.Tensor   # int32, one per bin
    offsets: torch.Tensor  # uint64 stored as int64, one per bin
    permutes: torch.Tensor  # uint64 stored as int64, end - begin entries

    def numBin(self):
        return self.counts.numel()

    def binSize(self, b):
        return int(self.counts[b])

    def binOffset(self, b):
        return int(self.offsets[b])

    def permutation(self, i):
        return int(self.permutes[i])

    def rangeBegin(self):
        return self.begin

    def rangeEnd(self):
        return self.end


class LinkedCellList:
    """LinkedCellList<MemorySpace, double, NumSpaceDim> (core/src/Cabana_LinkedCellList.hpp),
    NumSpaceDim = len(grid_min): 3 (positions (p, 0..2)) or 2 (positions (p, 0..1))."""

    def __init__(self, positions, grid_delta, grid_min, grid_max, begin=0, end=None, handle=None, stream=None):
        nd = len(grid_min)
        if nd not in (2, 3) or len(grid_max) != nd or len(grid_delta) != nd:
            raise ValueError("grid_min / grid_max / grid_delta need 2 or 3 entries each")
        d3 = ctypes.c_double * 3
        nb = (ctypes.c_int32 * 3)()
        # bin counts: a 2D grid is counted as a 3D one with a single z cell
        pad = lambda v, fill: d3(*(list(v) + [fill] * (3 - nd)))  # noqa: E731
        self._min, self._max, self._delta = pad(grid_min, 0.0), pad(grid_max, 1.0), pad(grid_delta, 1.0)
        d2 = ctypes.c_double * 2
        self._grid2 = (d2(*grid_min), d2(*grid_max), d2(*grid_delta)) if nd == 2 else None
        L.check(L.lib().cgx_cartesian_num_bins(self._min, self._max, self._delta, nb))
        self._nbin = tuple(nb)[:nd]
        self._handle, self._stream = handle, stream
        self._sorted = False
        self.build(positions, begin, end)

    def build(self, positions, begin=0, end=None):
        """Rebin (LinkedCellList::build, Cabana_LinkedCellList.hpp:651-775):
        the grid stays, the particles [begin, end) of `positions` are binned
        again, and the list counts as not sorted."""
        n = positions.size if isinstance(positions, Slice) else positions.shape[0]
        end = n if end is None else end
        if not 0 <= begin <= end <= n:
            raise ValueError("need 0 <= begin <= end <= number of positions")
        total = self.totalBins()
        dev = positions.storage.device if isinstance(positions, Slice) else positions.device
        counts = torch.zeros(total, dtype=torch.int32, device=dev)
        offsets = torch.zeros(total, dtype=torch.int64, device=dev)
        permutes = torch.zeros(max(1, end - begin), dtype=torch.int64, device=dev)
        h = self._handle or L.default_handle()
        outs = (ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(offsets.data_ptr()),
                ctypes.c_void_p(permutes.data_ptr()), _stream(self._stream))
        desc = ctypes.byref(field_descriptor(positions))
        if self._grid2 is None:
            L.check(L.lib().cgx_linked_cell_build(h.ptr, desc, begin, end, self._min, self._max, self._delta, *outs))
        else:
            L.check(L.lib().cgx_linked_cell_build_2d(h.ptr, desc, begin, end, *self._grid2, *outs))
        self._data = BinningData(begin, end, counts, offsets, permutes[: end - begin])
        self._sorted = False
        self._particle_bins = None  # formed on first use (storeParticleBins)

    def numBin(self, d):
        return self._nbin[d]

    def totalBins(self):
        t = 1
        for b in self._nbin:
            t *= b
        return t

    def _ijk(self, ijk):
        # binSize(i, j[, k]) or binSize((i, j[, k])) -- the reference's
        # Kokkos::Array overload
        if len(ijk) == 1 and isinstance(ijk[0], (tuple, list)):
            ijk = tuple(ijk[0])
        if len(ijk) != len(self._nbin):
            raise ValueError(f"need {len(self._nbin)} cell indices")
        return ijk

    def cardinalBinIndex(self, *ijk):
        ijk = self._ijk(ijk)
        c = 0
        for d, x in enumerate(ijk):
            c = c * self._nbin[d] + x
        return c

    def binSize(self, *ijk):
        return self._data.binSize(self.cardinalBinIndex(*ijk))

    def binOffset(self, *ijk):
        return self._data.binOffset(self.cardinalBinIndex(*ijk))

    def permutation(self, i):
        return self._data.permutation(i)

    def binningData(self):
        return self._data

    def ijkBinIndex(self, cardinal):
        """The (i, j[, k]) of a cardinal bin index (k, then j, fastest)."""
        out = []
        for d in range(len(self._nbin) - 1, -1, -1):
            out.append(cardinal % self._nbin[d])
            cardinal //= self._nbin[d]
        return tuple(reversed(out))

    def numParticles(self):
        return self._data.end - self._data.begin

    def getParticleBegin(self):
        return self._data.begin

    def getParticleEnd(self):
        return self._data.end

    def rangeBegin(self):
        return self._data.begin

    def rangeEnd(self):
        return self._data.end

    def update(self, sorted):
        """Record whether the particles have been permuted into bin order
        (LinkedCellList::update); the per-particle bins follow."""
        self._sorted = bool(sorted)
        self._particle_bins = None

    def sorted(self):
        return self._sorted

    def storeParticleBins(self):
        """The bin of every binned particle (LinkedCellList::storeParticleBins,
        Cabana_LinkedCellList.hpp:778-787 and :800-823): indexed by the
        particle's position in bin order once sorted, else by its original
        index, both relative to begin."""
        d = self._data
        n = d.end - d.begin
        cells = torch.arange(d.counts.numel(), dtype=torch.int32, device=d.counts.device)
        in_order = torch.repeat_interleave(cells, d.counts.to(torch.int64), output_size=n)
        if self._sorted:
            self._particle_bins = in_order
        else:
            bins = torch.empty(n, dtype=torch.int32, device=d.counts.device)
            bins[d.permutes - d.begin] = in_order
            self._particle_bins = bins
        return self._particle_bins

    def getParticleBins(self):
        return self._particle_bins if self._particle_bins is not None else self.storeParticleBins()

    def getParticleBin(self, particle_index):
        if not self._data.begin <= particle_index < self._data.end:
            raise IndexError("particle outside the binned range")
        return int(self.getParticleBins()[particle_index - self._data.begin])


def createLinkedCellList(positions, grid_delta, grid_min, grid_max, begin=0, end=None, **kw):
    return LinkedCellList(positions, grid_delta, grid_min, grid_max, begin, end, **kw)


def _int_keys(keys):
    if keys.dtype.is_floating_point or keys.dtype == torch.bool:
        raise TypeError("keys must be an integer tensor (values within int32)")
    return keys.to(torch.int32).contiguous()


def _slice_keys(s):
    """The values of a rank-1 Slice as a contiguous tensor (the reference
    copies a key slice into a View first, copySliceToView,
    core/src/Cabana_Sort.hpp:459-545): element i sits at offset +
    soa_stride * (i / VL) + i % VL of the storage."""
    if s.comps != 1:
        raise ValueError("key slices must have one component per particle")
    i = torch.arange(s.size, device=s.storage.device)
    idx = s.offset + (i // s.vector_length) * s.soa_stride + i % s.vector_length
    return s.storage.reshape(-1)[idx]


def _bin_range(keys, nbin, begin, end, sort_within_bins, handle, stream):
    if isinstance(keys, Slice):
        keys = _slice_keys(keys)
    end = keys.shape[0] if end is None else end
    if nbin < 0:
        raise ValueError("nbin must be >= 0")
    keys = _int_keys(keys)
    counts = torch.zeros(nbin + 1, dtype=torch.int32, device=keys.device)
    offsets = torch.zeros(nbin + 1, dtype=torch.int64, device=keys.device)
    permutes = torch.zeros(max(1, end - begin), dtype=torch.int64, device=keys.device)
    h = handle or L.default_handle()
    L.check(L.lib().cgx_bin_by_key_range(h.ptr, ctypes.c_void_p(keys.data_ptr()), begin, end, nbin,
                                         1 if sort_within_bins else 0, ctypes.c_void_p(counts.data_ptr()),
                                         ctypes.c_void_p(offsets.data_ptr()), ctypes.c_void_p(permutes.data_ptr()),
                                         _stream(stream)))
    return BinningData(begin, end, counts, offsets, permutes[: end - begin])


def binByKey(keys, nbin, begin=0, end=None, handle=None, stream=None):
    """Cabana::binByKey (core/src/Cabana_Sort.hpp:411-443): nbin + 1 bins
    splitting [min, max] of keys[begin, end) evenly (Kokkos::BinOp1D; one key
    value per bin when max - min <= nbin); stable order inside a bin. `keys`
    is an integer tensor or a rank-1 Slice of an integer member."""
    return _bin_range(keys, nbin, begin, end, False, handle, stream)


def sortByKey(keys, begin=0, end=None, handle=None, stream=None):
    """Cabana::sortByKey (core/src/Cabana_Sort.hpp:364-393): BinOp1D bins with
    nbin = (end - begin) // 2, entries ordered by key inside each bin (so the
    permutation sorts by key; equal keys keep index order). `keys` is an
    integer tensor or a rank-1 Slice of an integer member."""
    if end is None:
        end = keys.size if isinstance(keys, Slice) else keys.shape[0]
    return _bin_range(keys, (end - begin) // 2, begin, end, True, handle, stream)


def binByIndex(keys, nbin, begin=0, end=None, handle=None, stream=None):
    """Bins given by number: keys[begin, end) in [0, nbin), nbin bins, stable
    order inside a bin (no reference counterpart; cgx_bin_by_key)."""
    end = keys.shape[0] if end is None else end
    counts = torch.zeros(nbin, dtype=torch.int32, device=keys.device)
    offsets = torch.zeros(nbin, dtype=torch.int64, device=keys.device)
    permutes = torch.zeros(max(1, end - begin), dtype=torch.int64, device=keys.device)
    keys = keys.to(torch.int32).contiguous()
    h = handle or L.default_handle()
    L.check(L.lib().cgx_bin_by_key(h.ptr, ctypes.c_void_p(keys.data_ptr()), begin, end, nbin,
                                   ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(offsets.data_ptr()),
                                   ctypes.c_void_p(permutes.data_ptr()), _stream(stream)))
    return BinningData(begin, end, counts, offsets, permutes[: end - begin])


def _ncomp(x):
    if isinstance(x, Slice):
        return x.comps
    return 1 if x.dim() == 1 else int(x[0].numel())


def _move_descriptor(f):
    """cgx_field for permute, which moves elements bit for bit: an integer
    tensor travels as the float type of its element size (int32 as float32,
    int64 as float64), as the reference permutes int members with the rest of
    the AoSoA."""
    t = f.storage if isinstance(f, Slice) else f
    if isinstance(t, torch.Tensor) and not t.dtype.is_floating_point:
        if t.dtype == torch.bool or t.element_size() not in (4, 8):
            raise TypeError(f"permute moves 4- or 8-byte elements; got {t.dtype}")
        as_float = t.view(torch.float32 if t.element_size() == 4 else torch.float64)
        if isinstance(f, Slice):
            return Slice(as_float, f.offset, f.vector_length, f.soa_stride, f.comps, f.size).descriptor()
        return field_descriptor(as_float)
    return field_descriptor(f)


def permute(binning, *fields, handle=None, stream=None):
    """In-place permute of every field over the binning's range (float32,
    float64, int32 or int64 tensors, or Slices)."""
    data = binning.binningData() if isinstance(binning, LinkedCellList) else binning
    if isinstance(binning, LinkedCellList):
        # permute(LinkedCellList&, ...) marks the list sorted
        # (Cabana_LinkedCellList.hpp:1130-1146)
        binning.update(True)
    if data.end == data.begin or not fields:
        return
    n = len(fields)
    descs = (L.CgxField * n)(*[_move_descriptor(f) for f in fields])
    nc = (ctypes.c_int32 * n)(*[_ncomp(f) for f in fields])
    h = handle or L.default_handle()
    L.check(L.lib().cgx_permute(h.ptr, ctypes.c_void_p(data.permutes.data_ptr()), data.begin, data.end, descs, nc, n,
                                _stream(stream)))


def permute_by(perm, *fields, handle=None, stream=None):
    """Apply a gather permutation (sorted[i] = old[perm[i]]) to whole fields."""
    n_pts = perm.numel()
    bd = BinningData(0, n_pts, torch.empty(0), torch.empty(0), perm)
    permute(bd, *fields, handle=handle, stream=stream)
