"""cgx_bin_by_key_static: key binning for callers that may not let a library
allocate device memory (hosts whose device memory is owned by another
allocator, or loops where an allocation and the synchronisation it can bring
are not allowed). It works out of a fixed scratch array compiled into
libcgx. These checks call it through the C ABI and compare it, bit for bit,
with cgx_bin_by_key on two calls in a row -- the second call finds the first
call's leftovers in the shared scratch, so it also shows that the entry point
clears what it needs. This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from cabana_gb300 import _lib as L
from cabana_gb300 import core as C

pytestmark = pytest.mark.gpu


def _static_bin(keys, nbin, begin, end):
    n = end - begin
    counts = torch.zeros(nbin, dtype=torch.int32, device="cuda")
    offsets = torch.zeros(nbin, dtype=torch.int64, device="cuda")
    permutes = torch.zeros(max(1, n), dtype=torch.int64, device="cuda")
    st = L.lib().cgx_bin_by_key_static(ctypes.c_void_p(keys.data_ptr()), begin, end, nbin,
                                       ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(offsets.data_ptr()),
                                       ctypes.c_void_p(permutes.data_ptr()),
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    L.check(st)
    return counts, offsets, permutes[:n]


def test_static_scratch_binning_matches_allocating_entry_point():
    rng = np.random.default_rng(21)
    cases = [(200000, 5000, 0, 200000), (150000, 777, 1234, 140000)]  # two calls in a row, different sizes
    for n, nbin, begin, end in cases:
        keys = torch.tensor(rng.integers(0, nbin, size=n).astype(np.int32), device="cuda")
        counts, offsets, permutes = _static_bin(keys, nbin, begin, end)
        ref = C.binByIndex(keys, nbin, begin, end)
        torch.cuda.synchronize()
        assert torch.equal(counts, ref.counts)
        assert torch.equal(offsets, ref.offsets)
        assert torch.equal(permutes, ref.permutes)


def test_static_scratch_rejects_oversized_problems():
    keys = torch.zeros(4, dtype=torch.int32, device="cuda")
    counts = torch.zeros(4, dtype=torch.int32, device="cuda")
    offsets = torch.zeros(4, dtype=torch.int64, device="cuda")
    perm = torch.zeros(4, dtype=torch.int64, device="cuda")
    too_many = L.CGX_ERR_INVALID_ARG
    st = L.lib().cgx_bin_by_key_static(ctypes.c_void_p(keys.data_ptr()), 0, 262145, 4,
                                       ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(offsets.data_ptr()),
                                       ctypes.c_void_p(perm.data_ptr()), None)
    assert st == too_many
    assert b"CGX_STATIC_MAX_KEYS" in L.lib().cgx_last_error()
