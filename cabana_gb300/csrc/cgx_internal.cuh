// Internal device-side types and helpers shared by the cgx kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "../../include/cgx.h"

namespace cgx {

constexpr int kMaxOps = 8;
constexpr int kMaxKnot = 7;

// ---------------------------------------------------------------------------
// Point fields and grid arrays in device-friendly form.
// ---------------------------------------------------------------------------
struct DField {
    char* data;
    int32_t dtype;
    int32_t log2vl;  // log2(vector_length)
    int64_t soa_stride;
    int64_t comp_stride;
};

struct DArray {
    char* data;
    int32_t dtype;
    int32_t dofs;
};

struct DOp {
    int32_t kind;
    int32_t slot;  // index of the distinct target array (tiled kernels)
    double mult;
    float mult_f;  // the multiplier rounded to FP32 once, on the host
    int32_t reserved;
    DField x;
    DArray a;
};

// Geometry the kernels need, precomputed on the host exactly as
// evaluateSpline does (grid/src/Cabana_Grid_Splines.hpp:1293-1311):
// low = coordinates(Entity, {0,0,0}), dx = coordinates({1,1,1}) - low,
// rdx = 1 / dx.
struct DMesh {
    double low[3];
    double rdx[3];
    float rdx_f[3];
    int32_t ext[3];  // ghosted entity extents
};

__host__ __device__ inline int first_offset(int order) {
    return (order % 2 == 0) ? -(order / 2) : -((order - 1) / 2);
}

// Element offset of (p, 0); Kokkos Views (vector length 1) take the short path.
__device__ __forceinline__ int64_t field_base(const DField& f, int64_t p) {
    if (f.log2vl == 0) return p * f.soa_stride;
    return (p >> f.log2vl) * f.soa_stride + (p & ((int64_t(1) << f.log2vl) - 1));
}

__device__ __forceinline__ int64_t field_offset(const DField& f, int64_t p, int c) {
    return field_base(f, p) + int64_t(c) * f.comp_stride;
}

template <class T>
__device__ __forceinline__ T load_field(const DField& f, int64_t p, int c) {
    const int64_t o = field_offset(f, p, c);
    if (f.dtype == CGX_F64) return T(__ldg(reinterpret_cast<const double*>(f.data) + o));
    return T(__ldg(reinterpret_cast<const float*>(f.data) + o));
}

// Asynchronous 4-byte global -> shared copy (no register round trip); all
// copies issued by a thread complete at cp_async_wait_all().
__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem_src) : "memory");
}

// ---- bulk copies (TMA) tracked by a shared-memory mbarrier -----------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// One thread initialises the barrier (one arrival per phase), then the
// initialisation is made visible to the asynchronous (TMA) proxy.
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// Announce `bytes` more of bulk copies completing the current phase, then
// (after all copies are issued) the issuing thread's arrival.
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.expect_tx.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before its later bulk copies (asynchronous proxy).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// Bulk global -> shared copy: both addresses 16-byte aligned, bytes a
// multiple of 16. The caller orders earlier accesses of the destination
// (fence_proxy_async after the CTA barrier that ends them).
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Bulk shared -> global copy: both addresses 16-byte aligned, bytes a
// multiple of 16, tracked by the issuing thread's bulk async-group. The
// threads that wrote the source order their writes first (fence_proxy_async,
// then a CTA barrier).
__device__ __forceinline__ void bulk_copy_s2g(void* dst, const void* src, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }

// Wait until this thread's bulk stores have finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }

// Wait until this thread's bulk stores are complete.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }

// Extra floats per staging region of a point field: a dense field block is
// copied from the 16-byte boundary at or below its first element (up to 3
// floats early) and rounded up to whole 16-byte copies (up to 3 floats late).
constexpr int kOpSlack = 8;

// Polls of a bulk-copy barrier before a CTA gives up (CGX_ERR_TIMEOUT); far
// beyond any copy's latency.
constexpr int kMaxPolls = 1 << 22;

// Bounded wait for the phase of the given parity to complete. Returns false
// after `max_tries` polls (the caller records a timeout and stops).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int max_tries) {
    for (int t = 0; t < max_tries; ++t) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// L2 prefetch of particles [b, e) of a field stored densely per particle
// (vector length 1, components adjacent) by one bulk prefetch of the 16-byte
// blocks holding them, issued by thread 0; other layouts are left alone.
__device__ __forceinline__ void prefetch_field_range(const DField& f, int64_t b, int64_t e) {
    if (threadIdx.x != 0 || f.log2vl != 0 || f.comp_stride != 1 || e <= b) return;
    const int64_t elt = f.dtype == CGX_F64 ? 8 : 4;
    const uintptr_t lo = reinterpret_cast<uintptr_t>(f.data + b * f.soa_stride * elt) & ~uintptr_t(15);
    const uintptr_t hi = (reinterpret_cast<uintptr_t>(f.data + e * f.soa_stride * elt) + 15) & ~uintptr_t(15);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"(unsigned(hi - lo)) : "memory");
}

template <class T>
__device__ __forceinline__ void add_field(const DField& f, int64_t p, int c, T v) {
    const int64_t o = field_offset(f, p, c);
    if (f.dtype == CGX_F64) {
        double* ptr = reinterpret_cast<double*>(f.data) + o;
        *ptr += double(v);
    } else {
        float* ptr = reinterpret_cast<float*>(f.data) + o;
        *ptr += float(v);
    }
}

__device__ __forceinline__ int64_t node_index(const DMesh& m, int i, int j, int k) {
    return (int64_t(i) * m.ext[1] + j) * m.ext[2] + k;
}

template <class T>
__device__ __forceinline__ void atomic_add_array(const DArray& a, int64_t node, int dof, T v) {
    const int64_t o = node * a.dofs + dof;
    if (a.dtype == CGX_F64)
        atomicAdd(reinterpret_cast<double*>(a.data) + o, double(v));
    else
        atomicAdd(reinterpret_cast<float*>(a.data) + o, float(v));
}

template <class T>
__device__ __forceinline__ T load_array(const DArray& a, int64_t node, int dof) {
    const int64_t o = node * a.dofs + dof;
    if (a.dtype == CGX_F64) return T(reinterpret_cast<const double*>(a.data)[o]);
    return T(reinterpret_cast<const float*>(a.data)[o]);
}

// ---------------------------------------------------------------------------
// Spline<N> weights.
//
// Double form: the reference arithmetic of Splines.hpp:122-452 applied to
// the logical coordinate x0 (orders 0-3), Cox-de Boor for orders 4-6.
// Float form: the same polynomials evaluated in FP32 on the in-cell offset
// u = x0 - int(x0), formed beforehand from the double coordinate.
// ---------------------------------------------------------------------------

// b[j] = B_d(u + d - j): the d+1 uniform B-spline basis values on one cell.
template <int D, class T>
__device__ __forceinline__ void de_boor(T u, T* b) {
    b[0] = T(1);
#pragma unroll
    for (int d = 1; d <= D; ++d) {
        T nb[D + 1];
#pragma unroll
        for (int j = 0; j <= d; ++j) {
            T left = (j >= 1) ? (u + T(d - j)) * b[j - 1] : T(0);
            T right = (j <= d - 1) ? (T(1 + j) - u) * b[j] : T(0);
            nb[j] = (left + right) * (T(1) / T(d));
        }
#pragma unroll
        for (int j = 0; j <= d; ++j) b[j] = nb[j];
    }
}

template <int ORDER, class T>
struct SplineKernel {
    static constexpr int nk = ORDER + 1;

    // u: in-cell offset in [0, 1); r: 1/dx.
    __device__ __forceinline__ static void weights(T u, T r, T* w, T* g) {
        if constexpr (ORDER == 0) {
            w[0] = T(1);
            g[0] = T(0);
        } else if constexpr (ORDER == 1) {
            w[0] = T(1) - u;
            w[1] = u;
            g[0] = -r;
            g[1] = r;
        } else if constexpr (ORDER == 2 && sizeof(T) == 4) {
            // FP32: the same polynomials in factored form, free of the
            // cancellation of the expanded ones near the cell ends
            // (w0 = (1-u)^2 / 2, w2 = u^2 / 2), with the middle weight taken
            // from the partition of unity so the weights sum to 1 to within
            // one rounding, with no bias (grid mass is conserved).
            const T v = T(1) - u;
            w[0] = T(0.5) * v * v;
            w[2] = T(0.5) * u * u;
            w[1] = T(1) - (w[0] + w[2]);
            g[0] = -v * r;
            g[2] = u * r;
            g[1] = -(g[0] + g[2]);
        } else if constexpr (ORDER == 3 && sizeof(T) == 4) {
            // FP32 factored cubic B-spline: w0 = (1-u)^3 / 6, w3 = u^3 / 6,
            // w1 = 2/3 - u^2 (1 - u/2), and w2 from the partition of unity;
            // the gradient weights likewise sum to zero.
            const T v = T(1) - u;
            const T one_sixth = T(1.0 / 6.0);
            w[0] = one_sixth * v * v * v;
            w[3] = one_sixth * u * u * u;
            w[1] = T(2.0 / 3.0) - u * u * (T(1) - T(0.5) * u);
            w[2] = T(1) - ((w[0] + w[3]) + w[1]);
            g[0] = T(-0.5) * v * v * r;
            g[3] = T(0.5) * u * u * r;
            g[1] = u * (T(1.5) * u - T(2)) * r;
            g[2] = -((g[0] + g[3]) + g[1]);
        } else if constexpr (ORDER == 2) {
            const T nine_eights = T(9.0 / 8.0);
            T xn = u + T(0.5);
            w[0] = T(0.5) * xn * xn - T(1.5) * xn + nine_eights;
            g[0] = (xn - T(1.5)) * r;
            xn -= T(1);
            w[1] = -xn * xn + T(0.75);
            g[1] = (T(-2) * xn) * r;
            xn -= T(1);
            w[2] = T(0.5) * xn * xn + T(1.5) * xn + nine_eights;
            g[2] = (xn + T(1.5)) * r;
        } else if constexpr (ORDER == 3) {
            const T one_sixth = T(1.0 / 6.0);
            const T two_thirds = one_sixth * T(4);
            const T four_thirds = two_thirds * T(2);
            T xn = u + T(1);
            T xn2 = xn * xn;
            w[0] = -xn * xn2 * one_sixth + xn2 - T(2) * xn + four_thirds;
            g[0] = (T(-0.5) * xn * xn + T(2) * xn - T(2)) * r;
            xn -= T(1);
            xn2 = xn * xn;
            w[1] = T(0.5) * xn * xn2 - xn2 + two_thirds;
            g[1] = (T(1.5) * xn * xn - T(2) * xn) * r;
            xn -= T(1);
            xn2 = xn * xn;
            w[2] = T(-0.5) * xn * xn2 - xn2 + two_thirds;
            g[2] = (T(-1.5) * xn * xn - T(2) * xn) * r;
            xn -= T(1);
            xn2 = xn * xn;
            w[3] = xn * xn2 * one_sixth + xn2 + T(2) * xn + four_thirds;
            g[3] = (T(0.5) * xn * xn + T(2) * xn + T(2)) * r;
        } else {
            de_boor<ORDER, T>(u, w);
            T b[ORDER];
            de_boor<ORDER - 1, T>(u, b);
#pragma unroll
            for (int a = 0; a <= ORDER; ++a) {
                T left = (a >= 1) ? b[a - 1] : T(0);
                T right = (a <= ORDER - 1) ? b[a] : T(0);
                g[a] = (left - right) * r;
            }
        }
    }

    // Second derivatives of the knot weights with respect to the physical
    // coordinate (r2 = rdx^2): the derivative of `weights`' gradient. For
    // degree n, d2/du2 B_n = B_{n-2}[a-2] - 2 B_{n-2}[a-1] + B_{n-2}[a].
    // Orders 0 and 1 are piecewise constant / linear: zero almost everywhere.
    __device__ __forceinline__ static void hessian(T u, T r2, T* h) {
        if constexpr (ORDER <= 1) {
#pragma unroll
            for (int a = 0; a < nk; ++a) h[a] = T(0);
        } else if constexpr (ORDER == 2) {
            h[0] = r2;
            h[1] = T(-2) * r2;
            h[2] = r2;
        } else if constexpr (ORDER == 3) {
            h[0] = (T(1) - u) * r2;
            h[1] = (T(3) * u - T(2)) * r2;
            h[2] = (T(1) - T(3) * u) * r2;
            h[3] = u * r2;
        } else {
            T b[ORDER - 1];
            de_boor<ORDER - 2, T>(u, b);
#pragma unroll
            for (int a = 0; a <= ORDER; ++a) {
                const T l2 = (a >= 2) ? b[a - 2] : T(0);
                const T l1 = (a >= 1 && a - 1 <= ORDER - 2) ? b[a - 1] : T(0);
                const T l0 = (a <= ORDER - 2) ? b[a] : T(0);
                h[a] = (l2 - T(2) * l1 + l0) * r2;
            }
        }
    }
};

// Reference mapping in double: x0 = (xp - low) * rdx (+ 0.5 on the dual grid
// of even orders), rounded step by step with no contraction so the stencil
// index is bit-identical to the reference's.
template <int ORDER>
__device__ __forceinline__ double logical_coord(double xp, double low, double rdx) {
    double t = __dmul_rn(__dsub_rn(xp, low), rdx);
    if constexpr (ORDER % 2 == 0) t = __dadd_rn(t, 0.5);
    return t;
}

// Stencil base (first node index) and in-cell offset from the double
// logical coordinate, as Spline<N>::stencil / value do: int truncation.
template <int ORDER, class T>
__device__ __forceinline__ void base_and_offset(double x0, int& base, T& u) {
    const int c = static_cast<int>(x0);
    base = c + first_offset(ORDER);
    u = T(x0 - double(c));
}

// The mapping t = x * rdx + c0 of one dimension in integer form, for the
// FP32 kernels: rdx = r * 2^e with r a 64-bit integer (its leading bit set)
// and c = c0 * 2^32 rounded to an integer (see fixed_map).
struct FixedMap {
    uint64_t r;
    int64_t c;
    int32_t e;
    int32_t reserved;
};

// Host side: the FixedMap of rdx and c0. Valid for |c0| < 2^28 (the caller
// checks fixed_map_ok): then every t in [0, 2^29) has |x * rdx| < 2^30 and
// the 32.32 sum cannot overflow.
inline FixedMap fixed_map(double rdx, double c0) {
    FixedMap f;
    int k = 0;
    const double m = frexp(rdx, &k);  // rdx = m * 2^k, m in [0.5, 1)
    f.r = static_cast<uint64_t>(ldexp(m, 64));
    f.e = k - 64;
    f.c = static_cast<int64_t>(llround(ldexp(c0, 32)));
    f.reserved = 0;
    return f;
}

inline bool fixed_map_ok(double c0) { return std::fabs(c0) < 268435456.0; }

// Cell index and in-cell offset of t = x * rdx + c0 with integer
// operations only (no double-precision arithmetic, which runs at 1/64 of the
// FP32 rate on this part): x = m * 2^(ex - 1075), so x * rdx * 2^32 is the
// high half of (m * 2^11) * r, shifted by ex + e - 990, then c is added in
// 32.32 fixed point. The offset keeps 32 fraction bits and is truncated to
// FP32 toward zero (always < 1). The integer part of x * rdx * 2^32 is
// exact up to the truncation of the product (t is rounded differently from
// a double evaluation only in its last bits). Returns false for t < 0,
// t >= 2^30, infinities and NaN.
__device__ __forceinline__ bool fixed_logical(double x, const FixedMap& f, int& cell, float& u) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const int ex = int((b >> 52) & 0x7FF);
    long long t1 = 0;
    cell = 0;
    u = 0.0f;
    if (ex == 0x7FF) return false;  // infinity or NaN
    if (ex != 0) {                  // zero and subnormals map to 0
        const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
        const unsigned long long p = __umul64hi(m << 11, f.r);
        const int sh = ex + f.e - 990;
        if (sh >= 0) {
            if (sh > 62 || (p >> (62 - sh)) != 0) return false;  // |x * rdx| >= 2^30
            t1 = static_cast<long long>(p << sh);
        } else {
            t1 = sh < -63 ? 0 : static_cast<long long>(p >> (-sh));
        }
        if (b >> 63) t1 = -t1;
    }
    const long long t = t1 + f.c;
    if (t < 0 || t >= (1ll << 62)) return false;
    cell = int(t >> 32);
    u = __uint2float_rz(static_cast<unsigned int>(t & 0xFFFFFFFFll)) * 2.3283064365386963e-10f;  // * 2^-32
    return true;
}

// ---------------------------------------------------------------------------
// Error flag in device memory (one int per handle). Kernels never trap: a
// point whose stencil leaves the ghosted index space is skipped and the flag
// is raised.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void raise_error(int* flag, int code) {
    if (flag) atomicOr(flag, 1 << code);
}

inline int log2_int(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

}  // namespace cgx
