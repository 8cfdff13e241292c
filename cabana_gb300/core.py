"""Cabana core binning API over torch CUDA tensors.

  LinkedCellList / createLinkedCellList  (core/src/Cabana_LinkedCellList.hpp:128-1146)
  BinningData                           (core/src/Cabana_Sort.hpp:37-136)
  binByKey                              (core/src/Cabana_Sort.hpp:164-226)
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
    def __init__(self, positions, grid_delta, grid_min, grid_max, begin=0, end=None, handle=None, stream=None):
        n = positions.size if isinstance(positions, Slice) else positions.shape[0]
        end = n if end is None else end
        d3 = ctypes.c_double * 3
        nb = (ctypes.c_int32 * 3)()
        self._min, self._max, self._delta = d3(*grid_min), d3(*grid_max), d3(*grid_delta)
        L.check(L.lib().cgx_cartesian_num_bins(self._min, self._max, self._delta, nb))
        self._nbin = tuple(nb)
        total = self._nbin[0] * self._nbin[1] * self._nbin[2]
        dev = positions.storage.device if isinstance(positions, Slice) else positions.device
        counts = torch.zeros(total, dtype=torch.int32, device=dev)
        offsets = torch.zeros(total, dtype=torch.int64, device=dev)
        permutes = torch.zeros(max(1, end - begin), dtype=torch.int64, device=dev)
        h = handle or L.default_handle()
        L.check(L.lib().cgx_linked_cell_build(h.ptr, ctypes.byref(field_descriptor(positions)), begin, end,
                                              self._min, self._max, self._delta,
                                              ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(offsets.data_ptr()),
                                              ctypes.c_void_p(permutes.data_ptr()), _stream(stream)))
        self._data = BinningData(begin, end, counts, offsets, permutes[: end - begin])

    def numBin(self, d):
        return self._nbin[d]

    def totalBins(self):
        return self._nbin[0] * self._nbin[1] * self._nbin[2]

    def cardinalBinIndex(self, i, j, k):
        return (i * self._nbin[1] + j) * self._nbin[2] + k

    def binSize(self, i, j, k):
        return self._data.binSize(self.cardinalBinIndex(i, j, k))

    def binOffset(self, i, j, k):
        return self._data.binOffset(self.cardinalBinIndex(i, j, k))

    def permutation(self, i):
        return self._data.permutation(i)

    def binningData(self):
        return self._data


def createLinkedCellList(positions, grid_delta, grid_min, grid_max, begin=0, end=None, **kw):
    return LinkedCellList(positions, grid_delta, grid_min, grid_max, begin, end, **kw)


def binByKey(keys, nbin, begin=0, end=None, handle=None, stream=None):
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


def permute(binning, *fields, handle=None, stream=None):
    """In-place permute of every field over the binning's range."""
    data = binning.binningData() if isinstance(binning, LinkedCellList) else binning
    if data.end == data.begin or not fields:
        return
    n = len(fields)
    descs = (L.CgxField * n)(*[field_descriptor(f) for f in fields])
    nc = (ctypes.c_int32 * n)(*[_ncomp(f) for f in fields])
    h = handle or L.default_handle()
    L.check(L.lib().cgx_permute(h.ptr, ctypes.c_void_p(data.permutes.data_ptr()), data.begin, data.end, descs, nc, n,
                                _stream(stream)))


def permute_by(perm, *fields, handle=None, stream=None):
    """Apply a gather permutation (sorted[i] = old[perm[i]]) to whole fields."""
    n_pts = perm.numel()
    bd = BinningData(0, n_pts, torch.empty(0), torch.empty(0), perm)
    permute(bd, *fields, handle=handle, stream=stream)
