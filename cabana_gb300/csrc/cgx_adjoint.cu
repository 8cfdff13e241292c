// Position adjoint of p2g / g2p (no counterpart in the reference).
//
// Every forward operator is bilinear in a point field s and a grid array A
// with node weights W_n(x) or their gradients dW_n/dx_d
// (grid/src/Cabana_Grid_Interpolation.hpp:53-788), so the derivative of the
// scalar loss with respect to the point position is, per point,
//   dL/dx_e = mult * sum_n ( r_n dW_n/dx_e + sum_d q_n[d] d2W_n/(dx_e dx_d) )
// with r_n and q_n the pairing of s and A at node n (AdjointPattern). For
// cgx_p2g_adjoint s is the forward input field and A the cotangent of the
// forward array; for cgx_g2p_adjoint s is the cotangent of the forward
// output field and A the forward array. One thread per point, no atomics.
#include "cgx_kernels.cuh"

namespace cgx {

namespace {

__host__ __device__ inline int pattern_point_comps(int pattern) {
    switch (pattern) {
        case kAdjValue1: case kAdjGradA: return 1;
        case kAdjValue3: case kAdjGradS: return 3;
        default: return 9;
    }
}

template <int ORDER, class T>
__global__ void __launch_bounds__(256) adjoint_points_kernel(const __grid_constant__ AdjointParams prm) {
    using S = SplineKernel<ORDER, T>;
    constexpr int nk = S::nk;
    constexpr int U = ORDER <= 3 ? nk : 1;  // full unroll only for the hot orders
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < prm.num_point; p += stride) {
        int s[3];
        T w[3][nk], g[3][nk], h[3][nk];
        bool ok = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double xp = load_field<double>(prm.points, p, d);
            const double x0 = logical_coord<ORDER>(xp, prm.mesh.low[d], prm.mesh.rdx[d]);
            T u;
            base_and_offset<ORDER, T>(x0, s[d], u);
            ok &= (x0 >= 0.0) && (s[d] >= 0) && (s[d] + nk <= prm.mesh.ext[d]);
            const T r = sizeof(T) == 8 ? T(prm.mesh.rdx[d]) : T(prm.mesh.rdx_f[d]);
            S::weights(u, r, w[d], g[d]);
            S::hessian(u, r * r, h[d]);
        }
        if (!ok) {
            raise_error(prm.error_flag, CGX_ERR_OUT_OF_BOUNDS);
            continue;
        }
        T dx[3] = {T(0), T(0), T(0)};
        for (int t = 0; t < prm.n_terms; ++t) {
            const AdjointTerm& tm = prm.terms[t];
            const int pattern = tm.pattern;
            const int ns = pattern_point_comps(pattern);
            T sv[9];
#pragma unroll
            for (int c = 0; c < 9; ++c) sv[c] = c < ns ? load_field<T>(tm.s, p, c) : T(0);
            const bool one_dof = pattern == kAdjValue1 || pattern == kAdjGradS;
            T acc[3] = {T(0), T(0), T(0)};
#pragma unroll U
            for (int i = 0; i < nk; ++i)
#pragma unroll U
                for (int j = 0; j < nk; ++j)
#pragma unroll U
                    for (int k = 0; k < nk; ++k) {
                        const int64_t n = node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k);
                        T A[3];
                        A[0] = load_array<T>(tm.a, n, 0);
                        A[1] = one_dof ? T(0) : load_array<T>(tm.a, n, 1);
                        A[2] = one_dof ? T(0) : load_array<T>(tm.a, n, 2);
                        T r = T(0);
                        T q[3] = {T(0), T(0), T(0)};
                        switch (pattern) {
                            case kAdjValue1: r = sv[0] * A[0]; break;
                            case kAdjValue3: r = sv[0] * A[0] + sv[1] * A[1] + sv[2] * A[2]; break;
                            case kAdjGradA:
#pragma unroll
                                for (int d = 0; d < 3; ++d) q[d] = sv[0] * A[d];
                                break;
                            case kAdjGradS:
#pragma unroll
                                for (int d = 0; d < 3; ++d) q[d] = sv[d] * A[0];
                                break;
                            case kAdjTensor:
#pragma unroll
                                for (int b = 0; b < 3; ++b) q[b] = sv[b] * A[0] + sv[3 + b] * A[1] + sv[6 + b] * A[2];
                                break;
                            default:  // kAdjTensorT
#pragma unroll
                                for (int a = 0; a < 3; ++a)
                                    q[a] = sv[3 * a] * A[0] + sv[3 * a + 1] * A[1] + sv[3 * a + 2] * A[2];
                                break;
                        }
                        const T grad[3] = {g[0][i] * w[1][j] * w[2][k], w[0][i] * g[1][j] * w[2][k],
                                           w[0][i] * w[1][j] * g[2][k]};
                        const T h00 = h[0][i] * w[1][j] * w[2][k];
                        const T h11 = w[0][i] * h[1][j] * w[2][k];
                        const T h22 = w[0][i] * w[1][j] * h[2][k];
                        const T h01 = g[0][i] * g[1][j] * w[2][k];
                        const T h02 = g[0][i] * w[1][j] * g[2][k];
                        const T h12 = w[0][i] * g[1][j] * g[2][k];
                        acc[0] += r * grad[0] + h00 * q[0] + h01 * q[1] + h02 * q[2];
                        acc[1] += r * grad[1] + h01 * q[0] + h11 * q[1] + h12 * q[2];
                        acc[2] += r * grad[2] + h02 * q[0] + h12 * q[1] + h22 * q[2];
                    }
            const T mult = sizeof(T) == 8 ? T(tm.mult) : T(tm.mult_f);
#pragma unroll
            for (int e = 0; e < 3; ++e) dx[e] += mult * acc[e];
        }
#pragma unroll
        for (int e = 0; e < 3; ++e) add_field<T>(prm.points_bar, p, e, dx[e]);
    }
}

template <int ORDER>
cudaError_t launch_order(const AdjointParams& prm, bool fp64, int sms, cudaStream_t st) {
    const int threads = 256;
    int64_t blocks = (prm.num_point + threads - 1) / threads;
    if (blocks > int64_t(sms) * 16) blocks = int64_t(sms) * 16;
    if (blocks < 1) blocks = 1;
    if (fp64)
        adjoint_points_kernel<ORDER, double><<<int(blocks), threads, 0, st>>>(prm);
    else
        adjoint_points_kernel<ORDER, float><<<int(blocks), threads, 0, st>>>(prm);
    return cudaGetLastError();
}

}  // namespace

// Position adjoint of a value term from its gradient sums: grads holds, per
// point, D[e][c] = sum_n A_c(n) dW_n/dx_e at grads[p * 3 * ncomp + e * ncomp
// + c] (a ScalarGradientG2P / VectorGradientG2P of A with multiplier 1), so
// dL/dx_e += mult * sum_c s_c D[e][c].
__global__ void __launch_bounds__(256) adjoint_value_combine_kernel(DField points_bar, DField sf, const float* grads,
                                                                    int64_t n, int ncomp, float mult) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += stride) {
        float sv[3] = {0.0f, 0.0f, 0.0f};
        for (int c = 0; c < ncomp; ++c) sv[c] = load_field<float>(sf, p, c);
        const float* D = grads + p * 3 * ncomp;
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            float r = 0.0f;
            for (int c = 0; c < ncomp; ++c) r = fmaf(sv[c], D[e * ncomp + c], r);
            add_field<double>(points_bar, p, e, double(mult * r));
        }
    }
}

cudaError_t launch_adjoint_value_combine(const DField& points_bar, const DField& sf, const float* grads, int64_t n,
                                         int ncomp, float mult, int sms, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    int64_t b = (n + 255) / 256;
    if (b > int64_t(sms) * 16) b = int64_t(sms) * 16;
    adjoint_value_combine_kernel<<<int(b), 256, 0, st>>>(points_bar, sf, grads, n, ncomp, mult);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_points(const AdjointParams& prm, int order, bool fp64, int sms, cudaStream_t st) {
    if (prm.num_point == 0 || prm.n_terms == 0) return cudaSuccess;
    switch (order) {
        case 0: return launch_order<0>(prm, fp64, sms, st);
        case 1: return launch_order<1>(prm, fp64, sms, st);
        case 2: return launch_order<2>(prm, fp64, sms, st);
        case 3: return launch_order<3>(prm, fp64, sms, st);
        case 4: return launch_order<4>(prm, fp64, sms, st);
        case 5: return launch_order<5>(prm, fp64, sms, st);
        case 6: return launch_order<6>(prm, fp64, sms, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace cgx
