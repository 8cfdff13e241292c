// Point-parallel p2g / g2p kernels (one thread per point, global atomics),
// the halo fold / fill and the array fill.
//
// These restate what the reference's Kokkos CUDA path runs for
// Cabana::Grid::p2g / g2p (grid/src/Cabana_Grid_Interpolation.hpp:861-880,
// :1243-1262): full spline evaluation per point, then each functor scattering
// (atomically) into or gathering from the arrays. With T = double this is the
// "plain FP64" form; with T = float it is the order-agnostic fallback of the
// FP32 form, used when no tile ordering is supplied.
#include "cgx_kernels.cuh"

namespace cgx {

// Spline weights of point p on a 3D mesh (the SplineData of evaluateSpline,
// grid/src/Cabana_Grid_Splines.hpp:1280-1342); false when the stencil leaves
// the ghosted index space.
template <int ORDER, class T>
__device__ __forceinline__ bool weights_3d(const PointParams& prm, int64_t p, int* s, T (*w)[ORDER + 1],
                                           T (*g)[ORDER + 1]) {
    using S = SplineKernel<ORDER, T>;
    constexpr int nk = S::nk;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double xp = load_field<double>(prm.points, p, d);
        const double x0 = logical_coord<ORDER>(xp, prm.mesh.low[d], prm.mesh.rdx[d]);
        T u;
        base_and_offset<ORDER, T>(x0, s[d], u);
        ok &= (x0 >= 0.0) && (s[d] >= 0) && (s[d] + nk <= prm.mesh.ext[d]);
        if constexpr (sizeof(T) == 8)
            S::weights(u, prm.mesh.rdx[d], w[d], g[d]);
        else
            S::weights(u, prm.mesh.rdx_f[d], w[d], g[d]);
    }
    return ok;
}

// One P2G functor on point p (the functor bodies of Interpolation.hpp:
// 1324-1566 over P2G::value / gradient / divergence, :437-747), atomically.
template <int ORDER, class T>
__device__ __forceinline__ void p2g_apply(const PointParams& prm, const DOp& op, int64_t p, const int* s,
                                          const T (*w)[ORDER + 1], const T (*g)[ORDER + 1]) {
    constexpr int nk = ORDER + 1;
    constexpr int U = ORDER <= 3 ? nk : 1;  // full unroll only for the hot orders
    const T mult = sizeof(T) == 8 ? T(op.mult) : T(op.mult_f);
    switch (op.kind) {
        case CGX_SCALAR_VALUE_P2G: {
            const T pd = load_field<T>(op.x, p, 0) * mult;
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k)
                        atomic_add_array(op.a, node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k), 0,
                                         pd * w[0][i] * w[1][j] * w[2][k]);
            break;
        }
        case CGX_VECTOR_VALUE_P2G: {
            T pd[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) pd[d] = mult * load_field<T>(op.x, p, d);
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k) {
                        const int64_t n = node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k);
                        const T wijk = w[0][i] * w[1][j] * w[2][k];
#pragma unroll
                        for (int d = 0; d < 3; ++d) atomic_add_array(op.a, n, d, pd[d] * wijk);
                    }
            break;
        }
        case CGX_SCALAR_GRADIENT_P2G: {
            const T pd = load_field<T>(op.x, p, 0) * mult;
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k) {
                        const int64_t n = node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k);
                        atomic_add_array(op.a, n, 0, pd * g[0][i] * w[1][j] * w[2][k]);
                        atomic_add_array(op.a, n, 1, pd * w[0][i] * g[1][j] * w[2][k]);
                        atomic_add_array(op.a, n, 2, pd * w[0][i] * w[1][j] * g[2][k]);
                    }
            break;
        }
        case CGX_VECTOR_DIVERGENCE_P2G: {
            T pd[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) pd[d] = mult * load_field<T>(op.x, p, d);
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k) {
                        const T r = pd[0] * g[0][i] * w[1][j] * w[2][k] + pd[1] * w[0][i] * g[1][j] * w[2][k] +
                                    pd[2] * w[0][i] * w[1][j] * g[2][k];
                        atomic_add_array(op.a, node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k), 0, r);
                    }
            break;
        }
        case CGX_TENSOR_DIVERGENCE_P2G:
        case CGX_TENSOR_DIVERGENCE_T_P2G: {
            // pd[m][n]: the tensor entry paired with dW/dx_n for grid dof m
            const bool tr = op.kind == CGX_TENSOR_DIVERGENCE_T_P2G;
            T pd[3][3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) pd[a][b] = mult * load_field<T>(op.x, p, tr ? b * 3 + a : a * 3 + b);
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k) {
                        const int64_t n = node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k);
                        const T rg[3] = {g[0][i] * w[1][j] * w[2][k], w[0][i] * g[1][j] * w[2][k],
                                         w[0][i] * w[1][j] * g[2][k]};
#pragma unroll
                        for (int d0 = 0; d0 < 3; ++d0)
                            atomic_add_array(op.a, n, d0,
                                             rg[0] * pd[d0][0] + rg[1] * pd[d0][1] + rg[2] * pd[d0][2]);
                    }
            break;
        }
    }
}

// One G2P functor on point p (Interpolation.hpp:938-1182 over G2P::value /
// gradient / divergence, :53-364): x += multiplier * result.
template <int ORDER, class T>
__device__ __forceinline__ void g2p_apply(const PointParams& prm, const DOp& op, int64_t p, const int* s,
                                          const T (*w)[ORDER + 1], const T (*g)[ORDER + 1]) {
    constexpr int nk = ORDER + 1;
    constexpr int U = ORDER <= 3 ? nk : 1;
    const T mult = sizeof(T) == 8 ? T(op.mult) : T(op.mult_f);
    switch (op.kind) {
        case CGX_SCALAR_VALUE_G2P: {
            T result = T(0);
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k)
                        result += load_array<T>(op.a, node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k), 0) *
                                  w[0][i] * w[1][j] * w[2][k];
            add_field<T>(op.x, p, 0, mult * result);
            break;
        }
        case CGX_VECTOR_VALUE_G2P: {
            T result[3] = {T(0), T(0), T(0)};
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k) {
                        const int64_t n = node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k);
                        const T wijk = w[0][i] * w[1][j] * w[2][k];
#pragma unroll
                        for (int d = 0; d < 3; ++d) result[d] += load_array<T>(op.a, n, d) * wijk;
                    }
#pragma unroll
            for (int d = 0; d < 3; ++d) add_field<T>(op.x, p, d, mult * result[d]);
            break;
        }
        case CGX_SCALAR_GRADIENT_G2P: {
            T result[3] = {T(0), T(0), T(0)};
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k) {
                        const T f = load_array<T>(op.a, node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k), 0);
                        result[0] += f * g[0][i] * w[1][j] * w[2][k];
                        result[1] += f * w[0][i] * g[1][j] * w[2][k];
                        result[2] += f * w[0][i] * w[1][j] * g[2][k];
                    }
#pragma unroll
            for (int d = 0; d < 3; ++d) add_field<T>(op.x, p, d, mult * result[d]);
            break;
        }
        case CGX_VECTOR_GRADIENT_G2P:
        case CGX_VECTOR_GRADIENT_T_G2P: {
            // result[a][b] = sum dW/dx_a f_b, stored at (a, b) or transposed at (b, a)
            const bool tr = op.kind == CGX_VECTOR_GRADIENT_T_G2P;
            T result[3][3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) result[a][b] = T(0);
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k) {
                        const int64_t n = node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k);
                        const T rg[3] = {g[0][i] * w[1][j] * w[2][k], w[0][i] * g[1][j] * w[2][k],
                                         w[0][i] * w[1][j] * g[2][k]};
                        T v[3];
#pragma unroll
                        for (int d = 0; d < 3; ++d) v[d] = load_array<T>(op.a, n, d);
#pragma unroll
                        for (int a = 0; a < 3; ++a)
#pragma unroll
                            for (int b = 0; b < 3; ++b) result[a][b] += rg[a] * v[b];
                    }
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) add_field<T>(op.x, p, tr ? b * 3 + a : a * 3 + b, mult * result[a][b]);
            break;
        }
        case CGX_VECTOR_DIVERGENCE_G2P: {
            T result = T(0);
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k) {
                        const int64_t n = node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k);
                        result += load_array<T>(op.a, n, 0) * g[0][i] * w[1][j] * w[2][k] +
                                  load_array<T>(op.a, n, 1) * w[0][i] * g[1][j] * w[2][k] +
                                  load_array<T>(op.a, n, 2) * w[0][i] * w[1][j] * g[2][k];
                    }
            add_field<T>(op.x, p, 0, result * mult);
            break;
        }
    }
}

template <int ORDER, class T>
__global__ void __launch_bounds__(256) p2g_points_kernel(const __grid_constant__ PointParams prm) {
    constexpr int nk = ORDER + 1;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < prm.num_point; p += stride) {
        int s[3];
        T w[3][nk], g[3][nk];
        if (!weights_3d<ORDER, T>(prm, p, s, w, g)) {
            raise_error(prm.error_flag, CGX_ERR_OUT_OF_BOUNDS);
            continue;
        }
        for (int o = 0; o < prm.n_ops; ++o) p2g_apply<ORDER, T>(prm, prm.ops[o], p, s, w, g);
    }
}

template <int ORDER, class T>
__global__ void __launch_bounds__(256) g2p_points_kernel(const __grid_constant__ PointParams prm) {
    constexpr int nk = ORDER + 1;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < prm.num_point; p += stride) {
        int s[3];
        T w[3][nk], g[3][nk];
        if (!weights_3d<ORDER, T>(prm, p, s, w, g)) {
            raise_error(prm.error_flag, CGX_ERR_OUT_OF_BOUNDS);
            continue;
        }
        for (int o = 0; o < prm.n_ops; ++o) g2p_apply<ORDER, T>(prm, prm.ops[o], p, s, w, g);
    }
}

// Fused G2P then P2G per point (the g2p2g composition of
// benchmark/grid/Cabana_Grid_InterpolationPerformance.cpp:129-174): one
// spline evaluation, ops[0, n_g2p) gathered into their point fields, then
// ops[n_g2p, n_ops) scattered from point fields that may hold the values just
// gathered (same thread, program order).
template <int ORDER, class T>
__global__ void __launch_bounds__(256) g2p2g_points_kernel(const __grid_constant__ PointParams prm) {
    constexpr int nk = ORDER + 1;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < prm.num_point; p += stride) {
        int s[3];
        T w[3][nk], g[3][nk];
        if (!weights_3d<ORDER, T>(prm, p, s, w, g)) {
            raise_error(prm.error_flag, CGX_ERR_OUT_OF_BOUNDS);
            continue;
        }
        for (int o = 0; o < prm.n_g2p; ++o) g2p_apply<ORDER, T>(prm, prm.ops[o], p, s, w, g);
        for (int o = prm.n_g2p; o < prm.n_ops; ++o) p2g_apply<ORDER, T>(prm, prm.ops[o], p, s, w, g);
    }
}

// ---------------------------------------------------------------------------
// 2D meshes: the same two kernels over (i, j) stencils, an Array (i, j, dof)
// indexed as (i, j, 0, dof) with mesh.ext[2] == 1, vectors of 2 components
// and 2 x 2 tensors (the 2D specialisations of
// grid/src/Cabana_Grid_Interpolation.hpp:81-396 and :466-788).
// ---------------------------------------------------------------------------
template <int ORDER, class T>
__device__ __forceinline__ bool weights_2d(const PointParams& prm, int64_t p, int* s, T (*w)[ORDER + 1],
                                           T (*g)[ORDER + 1]) {
    using S = SplineKernel<ORDER, T>;
    constexpr int nk = S::nk;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        const double xp = load_field<double>(prm.points, p, d);
        const double x0 = logical_coord<ORDER>(xp, prm.mesh.low[d], prm.mesh.rdx[d]);
        T u;
        base_and_offset<ORDER, T>(x0, s[d], u);
        ok &= (x0 >= 0.0) && (s[d] >= 0) && (s[d] + nk <= prm.mesh.ext[d]);
        if constexpr (sizeof(T) == 8)
            S::weights(u, prm.mesh.rdx[d], w[d], g[d]);
        else
            S::weights(u, prm.mesh.rdx_f[d], w[d], g[d]);
    }
    return ok;
}

template <int ORDER, class T>
__global__ void __launch_bounds__(256) p2g_points_2d_kernel(const __grid_constant__ PointParams prm) {
    constexpr int nk = ORDER + 1;
    constexpr int U = ORDER <= 3 ? nk : 1;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < prm.num_point; p += stride) {
        int s[2];
        T w[2][nk], g[2][nk];
        if (!weights_2d<ORDER, T>(prm, p, s, w, g)) {
            raise_error(prm.error_flag, CGX_ERR_OUT_OF_BOUNDS);
            continue;
        }
        for (int o = 0; o < prm.n_ops; ++o) {
            const DOp& op = prm.ops[o];
            const T mult = sizeof(T) == 8 ? T(op.mult) : T(op.mult_f);
            const int kind = op.kind;
            // point data, premultiplied as the functors do (scalar: x * m,
            // vector / tensor: m * x)
            T pd[4] = {T(0), T(0), T(0), T(0)};
            if (kind == CGX_SCALAR_VALUE_P2G || kind == CGX_SCALAR_GRADIENT_P2G) {
                pd[0] = load_field<T>(op.x, p, 0) * mult;
            } else if (kind == CGX_VECTOR_VALUE_P2G || kind == CGX_VECTOR_DIVERGENCE_P2G) {
                pd[0] = mult * load_field<T>(op.x, p, 0);
                pd[1] = mult * load_field<T>(op.x, p, 1);
            } else {
                // pd[2 m + n]: the entry paired with dW/dx_n for grid dof m
                const bool tr = kind == CGX_TENSOR_DIVERGENCE_T_P2G;
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int b = 0; b < 2; ++b) pd[a * 2 + b] = mult * load_field<T>(op.x, p, tr ? b * 2 + a : a * 2 + b);
            }
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j) {
                    const int64_t n = node_index(prm.mesh, s[0] + i, s[1] + j, 0);
                    const T wij = w[0][i] * w[1][j];
                    const T rg[2] = {g[0][i] * w[1][j], w[0][i] * g[1][j]};
                    switch (kind) {
                        case CGX_SCALAR_VALUE_P2G: atomic_add_array(op.a, n, 0, pd[0] * wij); break;
                        case CGX_VECTOR_VALUE_P2G:
                            atomic_add_array(op.a, n, 0, pd[0] * wij);
                            atomic_add_array(op.a, n, 1, pd[1] * wij);
                            break;
                        case CGX_SCALAR_GRADIENT_P2G:
                            atomic_add_array(op.a, n, 0, pd[0] * rg[0]);
                            atomic_add_array(op.a, n, 1, pd[0] * rg[1]);
                            break;
                        case CGX_VECTOR_DIVERGENCE_P2G: atomic_add_array(op.a, n, 0, pd[0] * rg[0] + pd[1] * rg[1]); break;
                        default:
                            atomic_add_array(op.a, n, 0, rg[0] * pd[0] + rg[1] * pd[1]);
                            atomic_add_array(op.a, n, 1, rg[0] * pd[2] + rg[1] * pd[3]);
                            break;
                    }
                }
        }
    }
}

template <int ORDER, class T>
__global__ void __launch_bounds__(256) g2p_points_2d_kernel(const __grid_constant__ PointParams prm) {
    constexpr int nk = ORDER + 1;
    constexpr int U = ORDER <= 3 ? nk : 1;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < prm.num_point; p += stride) {
        int s[2];
        T w[2][nk], g[2][nk];
        if (!weights_2d<ORDER, T>(prm, p, s, w, g)) {
            raise_error(prm.error_flag, CGX_ERR_OUT_OF_BOUNDS);
            continue;
        }
        for (int o = 0; o < prm.n_ops; ++o) {
            const DOp& op = prm.ops[o];
            const T mult = sizeof(T) == 8 ? T(op.mult) : T(op.mult_f);
            const int kind = op.kind;
            const bool vec = !(kind == CGX_SCALAR_VALUE_G2P || kind == CGX_SCALAR_GRADIENT_G2P);
            // value sums V_c = sum W f_c and gradient sums D[m][c] = sum dW/dx_m f_c
            T V[2] = {T(0), T(0)}, D[2][2] = {{T(0), T(0)}, {T(0), T(0)}};
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j) {
                    const int64_t n = node_index(prm.mesh, s[0] + i, s[1] + j, 0);
                    const T wij = w[0][i] * w[1][j];
                    const T rg[2] = {g[0][i] * w[1][j], w[0][i] * g[1][j]};
                    const T f0 = load_array<T>(op.a, n, 0);
                    const T f1 = vec ? load_array<T>(op.a, n, 1) : T(0);
                    V[0] += f0 * wij;
                    V[1] += f1 * wij;
#pragma unroll
                    for (int m = 0; m < 2; ++m) {
                        D[m][0] += rg[m] * f0;
                        D[m][1] += rg[m] * f1;
                    }
                }
            switch (kind) {
                case CGX_SCALAR_VALUE_G2P: add_field<T>(op.x, p, 0, mult * V[0]); break;
                case CGX_VECTOR_VALUE_G2P:
                    add_field<T>(op.x, p, 0, mult * V[0]);
                    add_field<T>(op.x, p, 1, mult * V[1]);
                    break;
                case CGX_SCALAR_GRADIENT_G2P:
                    add_field<T>(op.x, p, 0, mult * D[0][0]);
                    add_field<T>(op.x, p, 1, mult * D[1][0]);
                    break;
                case CGX_VECTOR_GRADIENT_G2P:
                case CGX_VECTOR_GRADIENT_T_G2P: {
                    const bool tr = kind == CGX_VECTOR_GRADIENT_T_G2P;
#pragma unroll
                    for (int a = 0; a < 2; ++a)
#pragma unroll
                        for (int b = 0; b < 2; ++b) add_field<T>(op.x, p, tr ? b * 2 + a : a * 2 + b, mult * D[a][b]);
                    break;
                }
                case CGX_VECTOR_DIVERGENCE_G2P: add_field<T>(op.x, p, 0, (D[0][0] + D[1][1]) * mult); break;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Halo on one rank. A ghost entity has an owned partner when every
// dimension in which it lies outside the owned range is periodic
// (LocalGrid_impl.hpp:430-510 shared spaces; HaloBase.hpp unpack).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool halo_partner(const HaloParams& h, int i, int j, int k, int64_t& own) {
    const int idx[3] = {i, j, k};
    int o[3];
    bool ghost = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d >= h.dims) {
            o[d] = idx[d];
            continue;
        }
        const int hw = h.halo_width, nc = h.owned_cells[d];
        const int own_hi = h.periodic[d] ? hw + nc : hw + nc + h.node_extra;
        if (idx[d] >= hw && idx[d] < own_hi) {
            o[d] = idx[d];
            continue;
        }
        if (!h.periodic[d]) return false;
        ghost = true;
        int r = (idx[d] - hw) % nc;
        if (r < 0) r += nc;
        o[d] = hw + r;
    }
    own = (int64_t(o[0]) * h.ext[1] + o[1]) * h.ext[2] + o[2];
    return ghost;
}

// One thread per entity; only ghosts with an owned image do work. An owned
// image is never a ghost, so each mode reads and writes disjoint entries
// except for the atomic sums into owned images.
template <class T, int MODE>
__global__ void halo_kernel(const __grid_constant__ HaloParams h) {
    const int64_t total = int64_t(h.ext[0]) * h.ext[1] * h.ext[2];
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; n < total; n += stride) {
        const int k = int(n % h.ext[2]);
        const int j = int((n / h.ext[2]) % h.ext[1]);
        const int i = int(n / (int64_t(h.ext[1]) * h.ext[2]));
        int64_t own;
        if (!halo_partner(h, i, j, k, own)) continue;
        T* a = reinterpret_cast<T*>(h.data);
        for (int c = 0; c < h.dofs; ++c) {
            T* ghost = a + n * h.dofs + c;
            T* image = a + own * h.dofs + c;
            if constexpr (MODE == kHaloGather) {
                *ghost = *image;
            } else if constexpr (MODE == kHaloScatterSum) {
                atomicAdd(image, *ghost);
            } else if constexpr (MODE == kHaloGatherAdd) {
                *ghost += *image;
            } else {
                atomicAdd(image, *ghost);
                *ghost = T(0);
            }
        }
    }
}

template <class T>
__global__ void fill_kernel(T* data, int64_t count, T value) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += stride) data[i] = value;
}

static int grid_blocks(int64_t work, int threads, int sms) {
    int64_t b = (work + threads - 1) / threads;
    const int64_t cap = int64_t(sms) * 16;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return int(b);
}

template <int ORDER>
static cudaError_t launch_points_order(const PointParams& prm, bool p2g, bool fp64, int sms, cudaStream_t st) {
    const int threads = 256;
    const int blocks = grid_blocks(prm.num_point, threads, sms);
    if (prm.dims == 2) {
        if (p2g) {
            if (fp64)
                p2g_points_2d_kernel<ORDER, double><<<blocks, threads, 0, st>>>(prm);
            else
                p2g_points_2d_kernel<ORDER, float><<<blocks, threads, 0, st>>>(prm);
        } else {
            if (fp64)
                g2p_points_2d_kernel<ORDER, double><<<blocks, threads, 0, st>>>(prm);
            else
                g2p_points_2d_kernel<ORDER, float><<<blocks, threads, 0, st>>>(prm);
        }
        return cudaGetLastError();
    }
    if (p2g) {
        if (fp64)
            p2g_points_kernel<ORDER, double><<<blocks, threads, 0, st>>>(prm);
        else
            p2g_points_kernel<ORDER, float><<<blocks, threads, 0, st>>>(prm);
    } else {
        if (fp64)
            g2p_points_kernel<ORDER, double><<<blocks, threads, 0, st>>>(prm);
        else
            g2p_points_kernel<ORDER, float><<<blocks, threads, 0, st>>>(prm);
    }
    return cudaGetLastError();
}

cudaError_t launch_points(const PointParams& prm, int order, bool p2g, bool fp64, int sms, cudaStream_t st) {
    if (prm.num_point == 0) return cudaSuccess;
    switch (order) {
        case 0: return launch_points_order<0>(prm, p2g, fp64, sms, st);
        case 1: return launch_points_order<1>(prm, p2g, fp64, sms, st);
        case 2: return launch_points_order<2>(prm, p2g, fp64, sms, st);
        case 3: return launch_points_order<3>(prm, p2g, fp64, sms, st);
        case 4: return launch_points_order<4>(prm, p2g, fp64, sms, st);
        case 5: return launch_points_order<5>(prm, p2g, fp64, sms, st);
        case 6: return launch_points_order<6>(prm, p2g, fp64, sms, st);
    }
    return cudaErrorInvalidValue;
}

template <int ORDER>
static cudaError_t launch_g2p2g_order(const PointParams& prm, bool fp64, int sms, cudaStream_t st) {
    const int threads = 256;
    const int blocks = grid_blocks(prm.num_point, threads, sms);
    if (fp64)
        g2p2g_points_kernel<ORDER, double><<<blocks, threads, 0, st>>>(prm);
    else
        g2p2g_points_kernel<ORDER, float><<<blocks, threads, 0, st>>>(prm);
    return cudaGetLastError();
}

cudaError_t launch_g2p2g_points(const PointParams& prm, int order, bool fp64, int sms, cudaStream_t st) {
    if (prm.num_point == 0) return cudaSuccess;
    switch (order) {
        case 0: return launch_g2p2g_order<0>(prm, fp64, sms, st);
        case 1: return launch_g2p2g_order<1>(prm, fp64, sms, st);
        case 2: return launch_g2p2g_order<2>(prm, fp64, sms, st);
        case 3: return launch_g2p2g_order<3>(prm, fp64, sms, st);
        case 4: return launch_g2p2g_order<4>(prm, fp64, sms, st);
        case 5: return launch_g2p2g_order<5>(prm, fp64, sms, st);
        case 6: return launch_g2p2g_order<6>(prm, fp64, sms, st);
    }
    return cudaErrorInvalidValue;
}

template <class T>
static cudaError_t launch_halo_t(const HaloParams& h, int mode, int blocks, cudaStream_t st) {
    switch (mode) {
        case kHaloGather: halo_kernel<T, kHaloGather><<<blocks, 256, 0, st>>>(h); break;
        case kHaloScatterSum: halo_kernel<T, kHaloScatterSum><<<blocks, 256, 0, st>>>(h); break;
        case kHaloGatherAdd: halo_kernel<T, kHaloGatherAdd><<<blocks, 256, 0, st>>>(h); break;
        case kHaloScatterClear: halo_kernel<T, kHaloScatterClear><<<blocks, 256, 0, st>>>(h); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_halo(const HaloParams& h, int mode, int sms, cudaStream_t st) {
    const int64_t total = int64_t(h.ext[0]) * h.ext[1] * h.ext[2];
    const int blocks = grid_blocks(total, 256, sms);
    if (h.dtype == CGX_F64) return launch_halo_t<double>(h, mode, blocks, st);
    return launch_halo_t<float>(h, mode, blocks, st);
}

cudaError_t launch_fill(void* data, int dtype, int64_t count, double value, int sms, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    const int blocks = grid_blocks(count, 256, sms);
    if (dtype == CGX_F64)
        fill_kernel<double><<<blocks, 256, 0, st>>>(reinterpret_cast<double*>(data), count, value);
    else
        fill_kernel<float><<<blocks, 256, 0, st>>>(reinterpret_cast<float*>(data), count, float(value));
    return cudaGetLastError();
}

}  // namespace cgx
