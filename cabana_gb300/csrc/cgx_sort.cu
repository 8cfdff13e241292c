// Binning: cell keys, a stable LSD radix sort of (key, index) pairs, scans,
// permutes and tile-major work lists.
//
// The reference builds LinkedCellList bins with a histogram, an exclusive
// scan and an atomic slot per particle (core/src/Cabana_LinkedCellList.hpp:
// 686-731); the atomic order inside a bin is nondeterministic on parallel
// backends. Here the permutation comes from a stable sort, so particles inside
// a bin keep ascending index order -- the reference's Serial-backend order --
// and the result is bit-reproducible.
#include <climits>

#include "cgx_kernels.cuh"

namespace cgx {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortWarps = kSortThreads / 32;

int blocks_for(int64_t work, int threads, int sms, int per_sm = 16) {
    int64_t b = (work + threads - 1) / threads;
    const int64_t cap = int64_t(sms) * per_sm;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return int(b);
}

// ---------------------------------------------------------------------------
// Exclusive scan of int32 counts -> uint64 offsets (reduce / scan / apply).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t block_exclusive_scan(uint64_t v, uint64_t* warp_sums, uint64_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint64_t s = (lane < int(blockDim.x >> 5)) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < int(blockDim.x >> 5)) warp_sums[lane] = s;
    }
    __syncthreads();
    total = warp_sums[(blockDim.x >> 5) - 1];
    const uint64_t warp_prefix = warp ? warp_sums[warp - 1] : 0;
    __syncthreads();
    return warp_prefix + x - v;
}

__global__ void scan_reduce_kernel(const int32_t* in, int64_t n, uint64_t* block_sums) {
    __shared__ uint64_t warp_sums[32];
    const int64_t base = int64_t(blockIdx.x) * kScanTile;
    uint64_t s = 0;
#pragma unroll
    for (int r = 0; r < kScanItems; ++r) {
        const int64_t i = base + int64_t(r) * kScanThreads + threadIdx.x;
        if (i < n) s += uint64_t(uint32_t(in[i]));
    }
    uint64_t total;
    block_exclusive_scan(s, warp_sums, total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void scan_block_sums_kernel(uint64_t* sums, int64_t nb, uint64_t* total_out) {
    __shared__ uint64_t warp_sums[32];
    __shared__ uint64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
        const int64_t i = b0 + threadIdx.x;
        const uint64_t v = (i < nb) ? sums[i] : 0;
        uint64_t total;
        const uint64_t ex = block_exclusive_scan(v, warp_sums, total);
        const uint64_t c = carry;
        if (i < nb) sums[i] = c + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry = c + total;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

__global__ void scan_apply_kernel(const int32_t* in, int64_t n, const uint64_t* block_prefix, uint64_t* out) {
    __shared__ uint64_t warp_sums[32];
    const int64_t base = int64_t(blockIdx.x) * kScanTile;
    // Blocked arrangement: thread t owns items [t*kScanItems, (t+1)*kScanItems).
    uint64_t v[kScanItems];
    uint64_t s = 0;
#pragma unroll
    for (int r = 0; r < kScanItems; ++r) {
        const int64_t i = base + int64_t(threadIdx.x) * kScanItems + r;
        v[r] = (i < n) ? uint64_t(uint32_t(in[i])) : 0;
        s += v[r];
    }
    uint64_t total;
    uint64_t run = block_exclusive_scan(s, warp_sums, total) + block_prefix[blockIdx.x];
#pragma unroll
    for (int r = 0; r < kScanItems; ++r) {
        const int64_t i = base + int64_t(threadIdx.x) * kScanItems + r;
        if (i < n) out[i] = run;
        run += v[r];
    }
}

// ---------------------------------------------------------------------------
// LSD radix sort, 8 bits per pass, stable: within a pass, a block ranks its
// keys round by round in input order, warps by match_any and a per-digit
// prefix over the block's warps.
// ---------------------------------------------------------------------------
__global__ void radix_hist_kernel(const uint32_t* keys, int64_t n, int shift, uint32_t* hist, int64_t nblocks) {
    __shared__ uint32_t h[kRadix];
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x) h[d] = 0;
    __syncthreads();
    const int64_t base = int64_t(blockIdx.x) * kSortTile;
#pragma unroll 4
    for (int r = 0; r < kSortItems; ++r) {
        const int64_t i = base + int64_t(r) * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & (kRadix - 1)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x) hist[int64_t(d) * nblocks + blockIdx.x] = h[d];
}

__global__ void radix_scatter_kernel(const uint32_t* keys_in, const uint32_t* vals_in, int64_t n, int shift,
                                     const uint64_t* digit_offsets, int64_t nblocks, uint32_t* keys_out,
                                     uint32_t* vals_out, uint32_t val_base) {
    __shared__ uint64_t base[kRadix];
    __shared__ uint32_t running[kRadix];
    __shared__ uint32_t warp_hist[kSortWarps][kRadix];
    __shared__ uint32_t warp_base[kSortWarps][kRadix];
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x) {
        base[d] = digit_offsets[int64_t(d) * nblocks + blockIdx.x];
        running[d] = 0;
        for (int w = 0; w < kSortWarps; ++w) warp_hist[w][d] = 0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const int64_t tile_base = int64_t(blockIdx.x) * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        const int64_t i = tile_base + int64_t(r) * kSortThreads + threadIdx.x;
        const bool valid = i < n;
        uint32_t key = 0, val = 0;
        int digit = kRadix;  // sentinel for padding lanes
        if (valid) {
            key = keys_in[i];
            val = vals_in ? vals_in[i] : uint32_t(i) + val_base;
            digit = int((key >> shift) & (kRadix - 1));
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        const uint32_t rank = __popc(peers & lt_mask);
        if (valid && rank == 0) warp_hist[warp][digit] = __popc(peers);
        __syncthreads();
        for (int d = threadIdx.x; d < kRadix; d += blockDim.x) {
            uint32_t run = running[d];
#pragma unroll
            for (int w = 0; w < kSortWarps; ++w) {
                const uint32_t c = warp_hist[w][d];
                warp_base[w][d] = run;
                warp_hist[w][d] = 0;
                run += c;
            }
            running[d] = run;
        }
        __syncthreads();
        if (valid) {
            const uint64_t pos = base[digit] + warp_base[warp][digit] + rank;
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
    }
}

__global__ void widen_vals_kernel(const uint32_t* vals, int64_t n, uint64_t* out, uint64_t offset) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = uint64_t(vals[i]) + offset;
}

__global__ void iota_kernel(int64_t n, uint64_t* out, uint64_t offset) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) out[i] = uint64_t(i) + offset;
}

// Warp-aggregated increment of counts[key] (many points share a key in
// dense cells).
__device__ __forceinline__ void aggregated_count(int32_t* counts, int key, bool valid) {
    const int k = valid ? key : -1;
    const uint32_t peers = __match_any_sync(__activemask(), k);
    const int lane = threadIdx.x & 31;
    if (valid && lane == __ffs(peers) - 1) atomicAdd(counts + key, __popc(peers));
}

// CartesianGrid::locatePoint + cardinalCellIndex
// (core/src/impl/Cabana_CartesianGrid.hpp:171-182, :226-231; 2D :158-168,
// :233-238). With dims == 2 the host passes nx2 == 1 and the third
// coordinate is neither read nor binned, so the key is i * nx1 + j.
__global__ void cartesian_keys_kernel(DField pos, int dims, int64_t begin, int64_t end, double mn0, double mn1,
                                      double mn2, double r0, double r1, double r2, int nx0, int nx1, int nx2,
                                      uint32_t* keys, int32_t* counts, int* error_flag) {
    const int64_t n = end - begin;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    const int64_t nloop = (n + stride - 1) / stride * stride;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < nloop; t += stride) {
        const bool valid = t < n;
        int key = 0;
        if (valid) {
            const int64_t p = begin + t;
            const double mn[3] = {mn0, mn1, mn2}, rdx[3] = {r0, r1, r2};
            const int nx[3] = {nx0, nx1, nx2};
            int c[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (d >= dims) {
                    c[d] = 0;
                    continue;
                }
                c[d] = int(floor(__dmul_rn(__dsub_rn(load_field<double>(pos, p, d), mn[d]), rdx[d])));
                c[d] = (c[d] == nx[d]) ? c[d] - 1 : c[d];
                // The reference indexes out of bounds here: clamp to the edge
                // bin and set the flag word (the linked-cell build does not
                // synchronise to read it back).
                if (c[d] < 0 || c[d] >= nx[d]) {
                    raise_error(error_flag, CGX_ERR_OUT_OF_BOUNDS);
                    c[d] = c[d] < 0 ? 0 : nx[d] - 1;
                }
            }
            key = (c[0] * nx1 + c[1]) * nx2 + c[2];
            keys[t] = uint32_t(key);
        }
        aggregated_count(counts, key, valid);
    }
}

__global__ void key_hist_kernel(const int32_t* keys, int64_t begin, int64_t end, uint32_t* keys_out, int32_t* counts,
                                int32_t nbin, int* error_flag) {
    const int64_t n = end - begin;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    const int64_t nloop = (n + stride - 1) / stride * stride;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < nloop; t += stride) {
        bool valid = t < n;
        int key = 0;
        if (valid) {
            key = keys[begin + t];
            if (key < 0 || key >= nbin) {
                raise_error(error_flag, CGX_ERR_INVALID_ARG);
                key = key < 0 ? 0 : nbin - 1;
            }
            keys_out[t] = uint32_t(key);
        }
        aggregated_count(counts, key, valid);
    }
}

// Minimum and maximum of keys[begin, end) into minmax[0..1] (the reference's
// Impl::keyMinMax, core/src/Cabana_Sort.hpp:186-212), which the host set to
// (INT_MAX, INT_MIN): warp shuffles, then one atomic pair per warp.
__global__ void key_minmax_init_kernel(int* minmax) {
    minmax[0] = INT_MAX;
    minmax[1] = INT_MIN;
}

__global__ void key_minmax_kernel(const int32_t* keys, int64_t begin, int64_t end, int* minmax) {
    const int64_t n = end - begin;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    int lo = INT_MAX, hi = INT_MIN;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += stride) {
        const int k = keys[begin + t];
        lo = k < lo ? k : lo;
        hi = k > hi ? k : hi;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    if ((threadIdx.x & 31) == 0 && lo <= hi) {
        atomicMin(minmax, lo);
        atomicMax(minmax + 1, hi);
    }
}

// Kokkos::BinOp1D::bin of keys[begin, end): bin = int(mul * (key - kmin)),
// kept inside [0, nbins) against rounding, and counted per bin. The sort key
// written to keys_out is the bin, or key - kmin when the entries are also
// ordered by key inside their bins (bins grow with the key, so a stable sort
// by key - kmin orders by bin, then key, then index).
__global__ void key_bin1d_kernel(const int32_t* keys, int64_t begin, int64_t end, int kmin, double mul, int32_t nbins,
                                 int by_key, uint32_t* keys_out, int32_t* counts) {
    const int64_t n = end - begin;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    const int64_t nloop = (n + stride - 1) / stride * stride;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < nloop; t += stride) {
        const bool valid = t < n;
        int bin = 0;
        if (valid) {
            const int k = keys[begin + t];
            bin = int(mul * (double(k) - double(kmin)));
            bin = bin < 0 ? 0 : (bin >= nbins ? nbins - 1 : bin);
            keys_out[t] = by_key ? uint32_t(int64_t(k) - int64_t(kmin)) : uint32_t(bin);
        }
        aggregated_count(counts, bin, valid);
    }
}

// One thread per element: neighbouring lanes move the components of one
// particle, so the gathers read whole particles and the scratch copy is
// written and read contiguously. The element -> (particle, component) split
// uses 32-bit division whenever the element count allows it.
__device__ __forceinline__ void split_element(int64_t e, int ncomp, bool small, int64_t& i, int& c) {
    if (small) {
        const uint32_t q = uint32_t(e) / uint32_t(ncomp);
        i = q;
        c = int(uint32_t(e) - q * uint32_t(ncomp));
    } else {
        i = e / ncomp;
        c = int(e - i * ncomp);
    }
}

template <class T>
__global__ void permute_gather_kernel(const uint64_t* perm, int64_t begin, int64_t end, DField f, int ncomp,
                                      T* scratch) {
    const int64_t total = (end - begin) * ncomp;
    const bool small = total < (int64_t(1) << 32);
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    const T* data = reinterpret_cast<const T*>(f.data);
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += stride) {
        int64_t i;
        int c;
        split_element(e, ncomp, small, i, c);
        scratch[e] = data[field_offset(f, int64_t(perm[i]), c)];
    }
}

template <class T>
__global__ void permute_copy_back_kernel(int64_t begin, int64_t end, DField f, int ncomp, const T* scratch) {
    const int64_t total = (end - begin) * ncomp;
    const bool small = total < (int64_t(1) << 32);
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    T* data = reinterpret_cast<T*>(f.data);
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += stride) {
        int64_t i;
        int c;
        split_element(e, ncomp, small, i, c);
        data[field_offset(f, begin + i, c)] = scratch[e];
    }
}

// Tile-major key of each point: the base node of its stencil, grouped by
// tile. Uses the same double mapping as the interpolation kernels.
template <int ORDER>
__global__ void tile_keys_kernel(DMesh mesh, DField pts, int64_t n, int t0, int t1, int t2, int nt0, int nt1,
                                 int nt2, uint32_t* keys, int32_t* tile_counts) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    const int64_t nloop = (n + stride - 1) / stride * stride;
    const int tile[3] = {t0, t1, t2}, nt[3] = {nt0, nt1, nt2};
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < nloop; p += stride) {
        const bool valid = p < n;
        int tid = 0;
        if (valid) {
            int tc[3], lc[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double x0 = logical_coord<ORDER>(load_field<double>(pts, p, d), mesh.low[d], mesh.rdx[d]);
                int b = (x0 >= 0.0 && x0 < 2.0e9) ? int(x0) + first_offset(ORDER) : -1;
                b = b < 0 ? 0 : b;
                int t = b / tile[d];
                if (t >= nt[d]) t = nt[d] - 1;
                tc[d] = t;
                int l = b - t * tile[d];
                lc[d] = l < 0 ? 0 : (l >= tile[d] ? tile[d] - 1 : l);
            }
            tid = (tc[0] * nt[1] + tc[1]) * nt[2] + tc[2];
            const uint32_t local = uint32_t((lc[0] * tile[1] + lc[1]) * tile[2] + lc[2]);
            keys[p] = uint32_t(tid) * uint32_t(tile[0] * tile[1] * tile[2]) + local;
        }
        aggregated_count(tile_counts, tid, valid);
    }
}

__global__ void tile_chunks_kernel(const int64_t* tile_offsets, int64_t num_tiles, int64_t chunk, int32_t* chunks) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < num_tiles; t += stride) {
        const int64_t cnt = tile_offsets[t + 1] - tile_offsets[t];
        chunks[t] = int32_t((cnt + chunk - 1) / chunk);
    }
}

__global__ void tile_work_kernel(const int64_t* tile_offsets, int64_t num_tiles, int64_t chunk,
                                  const uint64_t* work_prefix, WorkItem* work) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < num_tiles; t += stride) {
        const int64_t b = tile_offsets[t], e = tile_offsets[t + 1];
        int64_t w = int64_t(work_prefix[t]);
        for (int64_t s = b; s < e; s += chunk, ++w) {
            WorkItem it;
            it.begin = s;
            it.end = (s + chunk < e) ? s + chunk : e;
            it.tile = int32_t(t);
            it.instance = 0;
            work[w] = it;
        }
    }
}

// Batched work lists: flat tile f of all instances belongs to instance i with
// tile_base[i] <= f < tile_base[i + 1]; offs[i] are that instance's tile
// offsets.
__device__ __forceinline__ int instance_of(const int64_t* tile_base, int n_inst, int64_t f) {
    int lo = 0, hi = n_inst;  // tile_base[lo] <= f < tile_base[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (tile_base[mid] <= f)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__global__ void batch_tile_chunks_kernel(const int64_t* const* offs, const int64_t* tile_base, int n_inst,
                                         int64_t total, int64_t chunk, int32_t* chunks) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t f = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; f < total; f += stride) {
        const int i = instance_of(tile_base, n_inst, f);
        const int64_t t = f - tile_base[i];
        const int64_t cnt = offs[i][t + 1] - offs[i][t];
        chunks[f] = int32_t((cnt + chunk - 1) / chunk);
    }
}

__global__ void batch_tile_work_kernel(const int64_t* const* offs, const int64_t* tile_base, int n_inst,
                                       int64_t total, int64_t chunk, const uint64_t* work_prefix, WorkItem* work) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t f = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; f < total; f += stride) {
        const int i = instance_of(tile_base, n_inst, f);
        const int64_t t = f - tile_base[i];
        const int64_t b = offs[i][t], e = offs[i][t + 1];
        int64_t w = int64_t(work_prefix[f]);
        for (int64_t s = b; s < e; s += chunk, ++w) {
            WorkItem it;
            it.begin = s;
            it.end = (s + chunk < e) ? s + chunk : e;
            it.tile = int32_t(t);
            it.instance = i;
            work[w] = it;
        }
    }
}

__global__ void u64_to_i64_tail_kernel(const uint64_t* offs, int64_t n, const uint64_t* total, int64_t* out) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i <= n; i += stride)
        out[i] = int64_t(i < n ? offs[i] : *total);
}

}  // namespace

size_t scan_scratch_bytes(int64_t n) {
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    return size_t(nb + 1) * sizeof(uint64_t) + 256;
}

cudaError_t exclusive_scan_counts(const int32_t* counts, int64_t n, uint64_t* offsets, uint64_t* total, void* scratch,
                                  int sms, cudaStream_t st) {
    (void)sms;
    if (n == 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(uint64_t), st);
        return cudaSuccess;
    }
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    uint64_t* block_sums = reinterpret_cast<uint64_t*>(scratch);
    scan_reduce_kernel<<<unsigned(nb), kScanThreads, 0, st>>>(counts, n, block_sums);
    scan_block_sums_kernel<<<1, 1024, 0, st>>>(block_sums, nb, total);
    scan_apply_kernel<<<unsigned(nb), kScanThreads, 0, st>>>(counts, n, block_sums, offsets);
    return cudaGetLastError();
}

size_t radix_sort_scratch_bytes(int64_t n) {
    const int64_t nb = (n + kSortTile - 1) / kSortTile;
    const int64_t hist_n = int64_t(kRadix) * nb;
    size_t bytes = 0;
    bytes += size_t(n) * 4 * 3;              // keys_b, vals_a, vals_b
    bytes += size_t(hist_n) * 4;             // hist
    bytes += size_t(hist_n) * 8;             // scanned hist
    bytes += scan_scratch_bytes(hist_n);     // scan scratch
    return bytes + 4 * 256;
}

static char* align_up(char* p, size_t a) {
    return reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + a - 1) / a * a);
}

cudaError_t radix_sort_pairs(uint32_t* keys_in, int64_t n, int key_bits, uint64_t* perm_out, const uint64_t* vals_in,
                             uint64_t val_offset, void* scratch, size_t scratch_bytes, int sms, cudaStream_t st) {
    (void)vals_in;
    (void)scratch_bytes;
    if (n == 0) return cudaSuccess;
    const int passes = (key_bits + kRadixBits - 1) / kRadixBits;
    if (passes == 0) {
        iota_kernel<<<blocks_for(n, 256, sms), 256, 0, st>>>(n, perm_out, val_offset);
        return cudaGetLastError();
    }
    const int64_t nb = (n + kSortTile - 1) / kSortTile;
    const int64_t hist_n = int64_t(kRadix) * nb;
    char* p = reinterpret_cast<char*>(scratch);
    uint32_t* keys_b = reinterpret_cast<uint32_t*>(p);
    p = align_up(p + size_t(n) * 4, 256);
    uint32_t* vals_a = reinterpret_cast<uint32_t*>(p);
    p = align_up(p + size_t(n) * 4, 256);
    uint32_t* vals_b = reinterpret_cast<uint32_t*>(p);
    p = align_up(p + size_t(n) * 4, 256);
    uint32_t* hist = reinterpret_cast<uint32_t*>(p);
    p = align_up(p + size_t(hist_n) * 4, 256);
    uint64_t* hoff = reinterpret_cast<uint64_t*>(p);
    p = align_up(p + size_t(hist_n) * 8, 256);
    void* scan_scratch = p;

    uint32_t* kin = keys_in;
    uint32_t* kout = keys_b;
    uint32_t* vin = nullptr;  // first pass: values are the indices
    uint32_t* vout = vals_a;
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = pass * kRadixBits;
        radix_hist_kernel<<<unsigned(nb), kSortThreads, 0, st>>>(kin, n, shift, hist, nb);
        cudaError_t e = exclusive_scan_counts(reinterpret_cast<const int32_t*>(hist), hist_n, hoff, nullptr,
                                              scan_scratch, sms, st);
        if (e != cudaSuccess) return e;
        radix_scatter_kernel<<<unsigned(nb), kSortThreads, 0, st>>>(kin, vin, n, shift, hoff, nb, kout, vout, 0u);
        // ping-pong
        uint32_t* kt = kin;
        kin = kout;
        kout = kt;
        vin = vout;
        vout = (vout == vals_a) ? vals_b : vals_a;
    }
    widen_vals_kernel<<<blocks_for(n, 256, sms), 256, 0, st>>>(vin, n, perm_out, val_offset);
    return cudaGetLastError();
}

cudaError_t cartesian_keys(const DField& pos, int dims, int64_t begin, int64_t end, const double* mn,
                           const double* rdx, const int32_t* nx, uint32_t* keys, int32_t* counts, int* error_flag,
                           cudaStream_t st, int sms) {
    const int64_t n = end - begin;
    if (n <= 0) return cudaSuccess;
    if ((dims != 2 && dims != 3) || (dims == 2 && nx[2] != 1)) return cudaErrorInvalidValue;
    cartesian_keys_kernel<<<blocks_for(n, 256, sms), 256, 0, st>>>(pos, dims, begin, end, mn[0], mn[1], mn[2],
                                                                    rdx[0], rdx[1], rdx[2], nx[0], nx[1], nx[2],
                                                                    keys, counts, error_flag);
    return cudaGetLastError();
}

cudaError_t key_minmax(const int32_t* keys, int64_t begin, int64_t end, int* minmax, cudaStream_t st, int sms) {
    key_minmax_init_kernel<<<1, 1, 0, st>>>(minmax);
    const int64_t n = end - begin;
    if (n > 0) key_minmax_kernel<<<blocks_for(n, 256, sms), 256, 0, st>>>(keys, begin, end, minmax);
    return cudaGetLastError();
}

cudaError_t key_bin1d(const int32_t* keys, int64_t begin, int64_t end, int kmin, double mul, int32_t nbins, bool by_key,
                      uint32_t* keys_out, int32_t* counts, cudaStream_t st, int sms) {
    const int64_t n = end - begin;
    if (n <= 0) return cudaSuccess;
    if (nbins < 1) return cudaErrorInvalidValue;
    key_bin1d_kernel<<<blocks_for(n, 256, sms), 256, 0, st>>>(keys, begin, end, kmin, mul, nbins, by_key ? 1 : 0,
                                                               keys_out, counts);
    return cudaGetLastError();
}

cudaError_t key_histogram(const int32_t* keys, int64_t begin, int64_t end, uint32_t* keys_out, int32_t* counts,
                          int32_t nbin, int* error_flag, cudaStream_t st, int sms) {
    const int64_t n = end - begin;
    if (n <= 0) return cudaSuccess;
    key_hist_kernel<<<blocks_for(n, 256, sms), 256, 0, st>>>(keys, begin, end, keys_out, counts, nbin, error_flag);
    return cudaGetLastError();
}

cudaError_t permute_field(const uint64_t* perm, int64_t begin, int64_t end, const DField& f, int ncomp, void* scratch,
                          cudaStream_t st, int sms) {
    const int64_t total = (end - begin) * ncomp;
    if (total <= 0) return cudaSuccess;
    const int blocks = blocks_for(total, 256, sms, 32);
    if (f.dtype == CGX_F64) {
        permute_gather_kernel<double><<<blocks, 256, 0, st>>>(perm, begin, end, f, ncomp,
                                                              reinterpret_cast<double*>(scratch));
        permute_copy_back_kernel<double><<<blocks, 256, 0, st>>>(begin, end, f, ncomp,
                                                                 reinterpret_cast<const double*>(scratch));
    } else {
        permute_gather_kernel<float><<<blocks, 256, 0, st>>>(perm, begin, end, f, ncomp,
                                                             reinterpret_cast<float*>(scratch));
        permute_copy_back_kernel<float><<<blocks, 256, 0, st>>>(begin, end, f, ncomp,
                                                                reinterpret_cast<const float*>(scratch));
    }
    return cudaGetLastError();
}

cudaError_t tile_keys(const DMesh& mesh, const DField& pts, int64_t n, int order, const int32_t* tile,
                      const int32_t* nt, uint32_t* keys, int32_t* tile_counts, cudaStream_t st, int sms) {
    if (n <= 0) return cudaSuccess;
    const int blocks = blocks_for(n, 256, sms);
#define CGX_TILE_KEYS(O)                                                                                          \
    tile_keys_kernel<O><<<blocks, 256, 0, st>>>(mesh, pts, n, tile[0], tile[1], tile[2], nt[0], nt[1], nt[2], keys, \
                                                tile_counts)
    switch (order) {
        case 0: CGX_TILE_KEYS(0); break;
        case 1: CGX_TILE_KEYS(1); break;
        case 2: CGX_TILE_KEYS(2); break;
        case 3: CGX_TILE_KEYS(3); break;
        case 4: CGX_TILE_KEYS(4); break;
        case 5: CGX_TILE_KEYS(5); break;
        case 6: CGX_TILE_KEYS(6); break;
        default: return cudaErrorInvalidValue;
    }
#undef CGX_TILE_KEYS
    return cudaGetLastError();
}

cudaError_t counts_to_int64_offsets(const int32_t* counts, int64_t n, int64_t* offsets, void* scratch, cudaStream_t st,
                                    int sms) {
    // offsets has n + 1 entries; the scan runs into a uint64 staging area
    // placed after the scan scratch.
    char* p = reinterpret_cast<char*>(scratch);
    uint64_t* total = reinterpret_cast<uint64_t*>(p);
    p = align_up(p + 8, 256);
    uint64_t* staging = reinterpret_cast<uint64_t*>(p);
    p = align_up(p + size_t(n) * 8, 256);
    cudaError_t e = exclusive_scan_counts(counts, n, staging, total, p, sms, st);
    if (e != cudaSuccess) return e;
    u64_to_i64_tail_kernel<<<blocks_for(n + 1, 256, sms), 256, 0, st>>>(staging, n, total, offsets);
    return cudaGetLastError();
}

cudaError_t build_work_items(const int64_t* tile_offsets, int64_t num_tiles, int64_t chunk, int64_t* work_prefix,
                             WorkItem* work, int64_t* work_count, void* scan_scratch, cudaStream_t st, int sms) {
    char* p = reinterpret_cast<char*>(scan_scratch);
    int32_t* chunk_counts = reinterpret_cast<int32_t*>(p);
    p = align_up(p + size_t(num_tiles) * 4, 256);
    tile_chunks_kernel<<<blocks_for(num_tiles, 256, sms), 256, 0, st>>>(tile_offsets, num_tiles, chunk, chunk_counts);
    cudaError_t e = exclusive_scan_counts(chunk_counts, num_tiles, reinterpret_cast<uint64_t*>(work_prefix),
                                          reinterpret_cast<uint64_t*>(work_count), p, sms, st);
    if (e != cudaSuccess) return e;
    tile_work_kernel<<<blocks_for(num_tiles, 256, sms), 256, 0, st>>>(
        tile_offsets, num_tiles, chunk, reinterpret_cast<const uint64_t*>(work_prefix), work);
    return cudaGetLastError();
}

cudaError_t build_batch_work_items(const int64_t* const* tile_offsets, const int64_t* tile_base, int n_inst,
                                   int64_t total_tiles, int64_t chunk, int64_t* work_prefix, WorkItem* work,
                                   int64_t* work_count, void* scan_scratch, cudaStream_t st, int sms) {
    char* p = reinterpret_cast<char*>(scan_scratch);
    int32_t* chunk_counts = reinterpret_cast<int32_t*>(p);
    p = align_up(p + size_t(total_tiles) * 4, 256);
    batch_tile_chunks_kernel<<<blocks_for(total_tiles, 256, sms), 256, 0, st>>>(tile_offsets, tile_base, n_inst,
                                                                                 total_tiles, chunk, chunk_counts);
    cudaError_t e = exclusive_scan_counts(chunk_counts, total_tiles, reinterpret_cast<uint64_t*>(work_prefix),
                                          reinterpret_cast<uint64_t*>(work_count), p, sms, st);
    if (e != cudaSuccess) return e;
    batch_tile_work_kernel<<<blocks_for(total_tiles, 256, sms), 256, 0, st>>>(
        tile_offsets, tile_base, n_inst, total_tiles, chunk, reinterpret_cast<const uint64_t*>(work_prefix), work);
    return cudaGetLastError();
}

}  // namespace cgx
