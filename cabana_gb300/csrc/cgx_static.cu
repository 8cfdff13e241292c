// Key binning that never allocates device memory.
//
// Some callers cannot let a library call cudaMalloc: code that runs inside a
// host application whose device memory is owned by another allocator (a
// pooled or budgeted framework that must account for every byte), and
// latency-sensitive loops where an allocation -- which may synchronise the
// device -- is not allowed. cgx_bin_by_key_static gives them the same result
// as cgx_bin_by_key using only a fixed scratch area compiled into this
// library: a file-scope __device__ array of kStaticScratchBytes, which every
// GPU that loads the library holds until the process exits.
//
// The array is shared by every call on a device and keeps the previous
// call's contents; everything that must start at zero is cleared inside the
// call. Calls that overlap on the GPU (other streams, or other host threads)
// race on the array and must be serialised by the caller.
//
// Host code may not use the array's name as a device address (on the host it
// is only a stand-in). The first call on each device, with that device
// current, resolves the real address with cudaGetSymbolAddress and caches it;
// make that first call before any stream capture.
#include <mutex>

#include "cgx_kernels.cuh"

namespace cgx {

namespace {

constexpr int64_t kStaticMaxKeys = CGX_STATIC_MAX_KEYS;
constexpr int64_t kStaticMaxBins = CGX_STATIC_MAX_BINS;
constexpr size_t kStaticScratchBytes = size_t(6) << 20;  // 6 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_static_mutex;
void* g_static_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (resolved once
// per device).
cudaError_t static_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return e;
        g_static_ptr[dev] = p;
    }
    *out = g_static_ptr[dev];
    return cudaSuccess;
}

char* align256(char* p) { return reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 255) / 256 * 256); }

cgx_status static_fail(cgx_status code, const char* msg) {
    set_last_error(msg);
    return code;
}

}  // namespace

}  // namespace cgx

using namespace cgx;

extern "C" cgx_status cgx_bin_by_key_static(const int32_t* keys, int64_t begin, int64_t end, int32_t nbin,
                                            int32_t* counts, uint64_t* offsets, uint64_t* permutes, void* stream) {
    if (begin < 0 || end < begin) return static_fail(CGX_ERR_INVALID_ARG, "need 0 <= begin <= end");
    if (nbin < 1) return static_fail(CGX_ERR_INVALID_ARG, "nbin must be >= 1");
    const int64_t n = end - begin;
    if (n > kStaticMaxKeys)
        return static_fail(CGX_ERR_INVALID_ARG,
                           "cgx_bin_by_key_static: more keys than CGX_STATIC_MAX_KEYS; use cgx_bin_by_key");
    if (nbin > kStaticMaxBins)
        return static_fail(CGX_ERR_INVALID_ARG,
                           "cgx_bin_by_key_static: more bins than CGX_STATIC_MAX_BINS; use cgx_bin_by_key");
    if ((!keys || !permutes) && n > 0) return static_fail(CGX_ERR_INVALID_ARG, "NULL keys / permutes");
    if (!counts || !offsets) return static_fail(CGX_ERR_INVALID_ARG, "NULL counts / offsets");

    // Layout of the scratch array: error flag, keys, then the sort / scan
    // scratch shared by the two phases (they run one after the other).
    const size_t sort_bytes = radix_sort_scratch_bytes(n);
    const size_t scan_bytes = scan_scratch_bytes(nbin);
    const size_t need = 256 + size_t(n) * 4 + 256 + (sort_bytes > scan_bytes ? sort_bytes : scan_bytes) + 256;
    if (need > kStaticScratchBytes)
        return static_fail(CGX_ERR_INVALID_ARG, "cgx_bin_by_key_static: problem needs more than the static scratch");

    void* base = nullptr;
    cudaError_t e = static_scratch(&base);
    if (e != cudaSuccess) return static_fail(CGX_ERR_CUDA, cudaGetErrorString(e));
    char* p = reinterpret_cast<char*>(base);
    int* flag = reinterpret_cast<int*>(p);
    p = align256(p + 256);
    uint32_t* k32 = reinterpret_cast<uint32_t*>(p);
    p = align256(p + size_t(n) * 4);
    void* scratch = p;

    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return static_fail(CGX_ERR_CUDA, cudaGetErrorString(e));
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return static_fail(CGX_ERR_CUDA, cudaGetErrorString(e));
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    // The previous call's contents are still there: clear what must start at 0.
    if ((e = cudaMemsetAsync(flag, 0, sizeof(int), st)) != cudaSuccess) return static_fail(CGX_ERR_CUDA, cudaGetErrorString(e));
    if ((e = cudaMemsetAsync(counts, 0, size_t(nbin) * sizeof(int32_t), st)) != cudaSuccess)
        return static_fail(CGX_ERR_CUDA, cudaGetErrorString(e));
    if ((e = key_histogram(keys, begin, end, k32, counts, nbin, flag, st, sms)) != cudaSuccess)
        return static_fail(CGX_ERR_CUDA, cudaGetErrorString(e));
    if ((e = exclusive_scan_counts(counts, nbin, offsets, nullptr, scratch, sms, st)) != cudaSuccess)
        return static_fail(CGX_ERR_CUDA, cudaGetErrorString(e));
    if (n > 0) {
        int bits = 0;
        while ((int64_t(1) << bits) < nbin) ++bits;
        if ((e = radix_sort_pairs(k32, n, bits, permutes, nullptr, uint64_t(begin), scratch, sort_bytes, sms, st)) !=
            cudaSuccess)
            return static_fail(CGX_ERR_CUDA, cudaGetErrorString(e));
    }
    int host_flag = 0;
    if ((e = cudaMemcpyAsync(&host_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return static_fail(CGX_ERR_CUDA, cudaGetErrorString(e));
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return static_fail(CGX_ERR_CUDA, cudaGetErrorString(e));
    if (host_flag & (1 << CGX_ERR_INVALID_ARG)) return static_fail(CGX_ERR_INVALID_ARG, "a key was outside [0, nbin)");
    return CGX_OK;
}
