// Tiled grid-to-point for particles in tile-major order (FP32 form).
//
// A persistent grid pulls work items (a tile and a contiguous run of its
// particles) from a device counter. The CTA stages the tile's node box of
// every source array in shared memory with coalesced loads, then each thread
// gathers for one particle at a time. All operators that read one array share
// a single pass over the stencil that forms, per dof n, the value sum
// V_n = sum W v_n and the gradient sums D_mn = sum d_m W v_n in factorised
// (tensor-product) order; each functor then takes its result from them:
//   ScalarValueG2P V_0, VectorValueG2P V_n, ScalarGradientG2P D_m0,
//   VectorGradientG2P D_mn, VectorDivergenceG2P sum_m D_mm
// (grid/src/Cabana_Grid_Interpolation.hpp:53-364, :938-1182).
// A point whose stencil leaves the box reads the Array directly, so the
// ordering never changes the result.
#include "cgx_kernels.cuh"

namespace cgx {

namespace {

constexpr int kThreads = 256;

template <int ORDER>
__device__ __forceinline__ bool form_point(const TiledParams& prm, const double* x, int* s, float* u) {
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double t = fma(x[d], prm.mesh.rdx[d], prm.c0[d]);
        int c;
        ok &= split_logical(t, c, u[d]);
        s[d] = c + first_offset(ORDER);
        ok &= (s[d] >= 0) && (s[d] + ORDER + 1 <= prm.mesh.ext[d]);
    }
    return ok;
}

// Gather sums for one array: V[n] = sum W v_n, D[m][n] = sum d_m W v_n.
template <int ORDER, int NDOF, bool GRAD, bool BOXED>
__device__ __forceinline__ void gather_sums(const TiledParams& prm, const TiledArray& ta, const float* box,
                                            const int* l, const int* s, const float (*w)[ORDER + 1],
                                            const float (*g)[ORDER + 1], float* V, float (*D)[3]) {
    constexpr int K = ORDER + 1;
    const int dofs = ta.a.dofs;
#pragma unroll
    for (int n = 0; n < NDOF; ++n) {
        V[n] = 0.0f;
#pragma unroll
        for (int m = 0; m < 3; ++m) D[m][n] = 0.0f;
    }
#pragma unroll
    for (int i = 0; i < K; ++i) {
        float Tww[NDOF], Tgw[NDOF], Twg[NDOF];
#pragma unroll
        for (int n = 0; n < NDOF; ++n) Tww[n] = Tgw[n] = Twg[n] = 0.0f;
#pragma unroll
        for (int j = 0; j < K; ++j) {
            float Sw[NDOF], Sg[NDOF];
#pragma unroll
            for (int n = 0; n < NDOF; ++n) Sw[n] = Sg[n] = 0.0f;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                float v[NDOF];
                if (BOXED) {
                    const int node = ((l[0] + i) * prm.box[1] + (l[1] + j)) * prm.box[2] + (l[2] + k);
#pragma unroll
                    for (int n = 0; n < NDOF; ++n) v[n] = box[node * dofs + n];
                } else {
                    const int64_t node = node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k);
#pragma unroll
                    for (int n = 0; n < NDOF; ++n) v[n] = load_array<float>(ta.a, node, n);
                }
#pragma unroll
                for (int n = 0; n < NDOF; ++n) {
                    Sw[n] = fmaf(w[2][k], v[n], Sw[n]);
                    if (GRAD) Sg[n] = fmaf(g[2][k], v[n], Sg[n]);
                }
            }
#pragma unroll
            for (int n = 0; n < NDOF; ++n) {
                Tww[n] = fmaf(w[1][j], Sw[n], Tww[n]);
                if (GRAD) {
                    Tgw[n] = fmaf(g[1][j], Sw[n], Tgw[n]);
                    Twg[n] = fmaf(w[1][j], Sg[n], Twg[n]);
                }
            }
        }
#pragma unroll
        for (int n = 0; n < NDOF; ++n) {
            V[n] = fmaf(w[0][i], Tww[n], V[n]);
            if (GRAD) {
                D[0][n] = fmaf(g[0][i], Tww[n], D[0][n]);
                D[1][n] = fmaf(w[0][i], Tgw[n], D[1][n]);
                D[2][n] = fmaf(w[0][i], Twg[n], D[2][n]);
            }
        }
    }
}

template <int NDOF>
__device__ __forceinline__ void apply_ops(const TiledParams& prm, int slot, int64_t p, const float* V,
                                          const float (*D)[3]) {
    for (int o = 0; o < prm.n_ops; ++o) {
        const DOp& op = prm.ops[o];
        if (op.slot != slot) continue;
        const float mult = float(op.mult);
        switch (op.kind) {
            case CGX_SCALAR_VALUE_G2P:
                add_field<float>(op.x, p, 0, mult * V[0]);
                break;
            case CGX_VECTOR_VALUE_G2P:
                if (NDOF >= 3) {
#pragma unroll
                    for (int d = 0; d < 3; ++d) add_field<float>(op.x, p, d, mult * V[d < NDOF ? d : 0]);
                }
                break;
            case CGX_SCALAR_GRADIENT_G2P:
#pragma unroll
                for (int d = 0; d < 3; ++d) add_field<float>(op.x, p, d, mult * D[d][0]);
                break;
            case CGX_VECTOR_GRADIENT_G2P:
                if (NDOF >= 3) {
#pragma unroll
                    for (int a = 0; a < 3; ++a)
#pragma unroll
                        for (int b = 0; b < 3; ++b) add_field<float>(op.x, p, a * 3 + b, mult * D[a][b < NDOF ? b : 0]);
                }
                break;
            case CGX_VECTOR_DIVERGENCE_G2P:
                if (NDOF >= 3) add_field<float>(op.x, p, 0, (D[0][0] + D[1][1 < NDOF ? 1 : 0] + D[2][2 < NDOF ? 2 : 0]) * mult);
                break;
        }
    }
}

template <int ORDER, int NDOF, bool GRAD>
__global__ void __launch_bounds__(kThreads, ORDER >= 3 ? 1 : 2)
    g2p_tiled_kernel(const __grid_constant__ TiledParams prm, int slot) {
    constexpr int K = ORDER + 1;
    extern __shared__ float smem[];
    __shared__ int item_idx;
    const int64_t nwork = *prm.work_count;
    const TiledArray& ta = prm.arrays[slot];
    while (true) {
        if (threadIdx.x == 0) item_idx = atomicAdd(prm.work_counter, 1);
        __syncthreads();
        const int64_t widx = item_idx;
        if (widx >= nwork) break;
        const WorkItem it = prm.work[widx];
        int origin[3];
        {
            const int t2 = it.tile % prm.num_tiles[2];
            const int t1 = (it.tile / prm.num_tiles[2]) % prm.num_tiles[1];
            const int t0 = it.tile / (prm.num_tiles[1] * prm.num_tiles[2]);
            origin[0] = t0 * prm.tile[0];
            origin[1] = t1 * prm.tile[1];
            origin[2] = t2 * prm.tile[2];
        }
        // Stage the node box of the source array (coalesced rows of k * dofs).
        {
            const int dofs = ta.a.dofs;
            const int row = prm.box[2] * dofs;
            const int count = prm.box_nodes * dofs;
            for (int e = threadIdx.x; e < count; e += blockDim.x) {
                const int r = e / row, c = e - r * row;
                const int bj = r % prm.box[1], bi = r / prm.box[1];
                const int bk = c / dofs, dof = c - bk * dofs;
                const int gi = origin[0] + bi, gj = origin[1] + bj, gk = origin[2] + bk;
                float v = 0.0f;
                if (gi < prm.mesh.ext[0] && gj < prm.mesh.ext[1] && gk < prm.mesh.ext[2])
                    v = load_array<float>(ta.a, node_index(prm.mesh, gi, gj, gk), dof);
                smem[e] = v;
            }
        }
        __syncthreads();

        // Software pipeline: the next particle's coordinates are loaded and
        // its output lines prefetched while the current one is computed.
        double xn[3] = {0.0, 0.0, 0.0};
        int64_t p = it.begin + threadIdx.x;
        if (p < it.end) {
#pragma unroll
            for (int d = 0; d < 3; ++d) xn[d] = load_field<double>(prm.points, p, d);
        }
        for (; p < it.end; p += blockDim.x) {
            double x[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) x[d] = xn[d];
            const int64_t pn = p + blockDim.x;
            if (pn < it.end) {
#pragma unroll
                for (int d = 0; d < 3; ++d) xn[d] = load_field<double>(prm.points, pn, d);
                for (int o = 0; o < prm.n_ops; ++o) {
                    if (prm.ops[o].slot != slot) continue;
                    const int kind = prm.ops[o].kind;
                    const int last = kind == CGX_VECTOR_GRADIENT_G2P ? 8
                                     : (kind == CGX_VECTOR_VALUE_G2P || kind == CGX_SCALAR_GRADIENT_G2P) ? 2 : 0;
                    prefetch_field(prm.ops[o].x, pn, 0);
                    if (last) prefetch_field(prm.ops[o].x, pn, last);
                }
            }
            int s[3];
            float u[3];
            if (!form_point<ORDER>(prm, x, s, u)) {
                raise_error(prm.error_flag, CGX_ERR_OUT_OF_BOUNDS);
                continue;
            }
            float w[3][K], g[3][K];
#pragma unroll
            for (int d = 0; d < 3; ++d) SplineKernel<ORDER, float>::weights(u[d], prm.mesh.rdx_f[d], w[d], g[d]);
            int l[3];
            bool inbox = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                l[d] = s[d] - origin[d];
                inbox &= (l[d] >= 0) && (l[d] + K <= prm.box[d]);
            }
            float V[NDOF], D[3][3];
            if (inbox)
                gather_sums<ORDER, NDOF, GRAD, true>(prm, ta, smem, l, s, w, g, V, D);
            else
                gather_sums<ORDER, NDOF, GRAD, false>(prm, ta, smem, l, s, w, g, V, D);
            apply_ops<NDOF>(prm, slot, p, V, D);
        }
        __syncthreads();
    }
}

template <int ORDER, int NDOF, bool GRAD>
cudaError_t launch_g2p(const TiledParams& prm, int slot, int sms, size_t smem, cudaStream_t st) {
    const void* fn = reinterpret_cast<const void*>(&g2p_tiled_kernel<ORDER, NDOF, GRAD>);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    g2p_tiled_kernel<ORDER, NDOF, GRAD><<<sms * per_sm, kThreads, smem, st>>>(prm, slot);
    return cudaGetLastError();
}

template <int ORDER>
cudaError_t launch_g2p_slot(const TiledParams& prm, int slot, int ndof, bool grad, int sms, size_t smem,
                            cudaStream_t st) {
    if (ndof == 3) return grad ? launch_g2p<ORDER, 3, true>(prm, slot, sms, smem, st)
                               : launch_g2p<ORDER, 3, false>(prm, slot, sms, smem, st);
    return grad ? launch_g2p<ORDER, 1, true>(prm, slot, sms, smem, st)
                : launch_g2p<ORDER, 1, false>(prm, slot, sms, smem, st);
}

}  // namespace

// Dofs gathered (1 or 3) and whether gradient sums are needed, from the
// operators that read one array.
void g2p_slot_need(const TiledParams& prm, int slot, int& ndof, bool& grad) {
    ndof = 1;
    grad = false;
    for (int o = 0; o < prm.n_ops; ++o) {
        if (prm.ops[o].slot != slot) continue;
        switch (prm.ops[o].kind) {
            case CGX_SCALAR_VALUE_G2P: break;
            case CGX_VECTOR_VALUE_G2P: ndof = 3; break;
            case CGX_SCALAR_GRADIENT_G2P: grad = true; break;
            case CGX_VECTOR_GRADIENT_G2P:
            case CGX_VECTOR_DIVERGENCE_G2P: ndof = 3; grad = true; break;
        }
    }
}

cudaError_t launch_g2p_tiled(const TiledParams& prm, int order, int slot, int sms, size_t smem, cudaStream_t st) {
    int ndof;
    bool grad;
    g2p_slot_need(prm, slot, ndof, grad);
    switch (order) {
        case 1: return launch_g2p_slot<1>(prm, slot, ndof, grad, sms, smem, st);
        case 2: return launch_g2p_slot<2>(prm, slot, ndof, grad, sms, smem, st);
        case 3: return launch_g2p_slot<3>(prm, slot, ndof, grad, sms, smem, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace cgx
