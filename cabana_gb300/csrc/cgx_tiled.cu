// Tiled p2g / g2p for particles in tile-major order (the FP32-compensated
// form).
//
// A persistent grid pulls work items (a tile and a contiguous run of its
// particles) from a device counter. For p2g a CTA accumulates the run into a
// shared-memory node box (the tile's base nodes plus the stencil reach) with
// two-sum compensation, then flushes the box to the Array with one atomic per
// node and dof. For g2p the CTA stages the node box of every source array in
// shared memory and gathers from it. A point whose stencil leaves the box
// (one filed under the wrong tile) goes straight to global memory, so the
// ordering only affects speed, never the result.
//
// Same arithmetic as Cabana::Grid::P2G / G2P (grid/src/Cabana_Grid_
// Interpolation.hpp:53-747) in FP32 with the cell index and in-cell offset
// formed in double.
#include "cgx_kernels.cuh"

namespace cgx {

namespace {

// Compensated accumulation into a (sum, comp) pair held in shared memory.
// atomicAdd returns the value it replaced, so the rounding error of that
// very addition can be recovered exactly (TwoSum) and kept in `comp`.
__device__ __forceinline__ void comp_add(float* sum, float* comp, float v) {
    const float old = atomicAdd(sum, v);
    const float s = old + v;
    const float bp = s - old;
    const float e = (old - (s - bp)) + (v - bp);
    if (e != 0.0f) atomicAdd(comp, e);
}

struct Box {
    int origin[3];  // first base node of the tile
    int box[3];
};

__device__ __forceinline__ void tile_origin(const TiledParams& prm, int tile, int* origin) {
    const int t2 = tile % prm.num_tiles[2];
    const int t1 = (tile / prm.num_tiles[2]) % prm.num_tiles[1];
    const int t0 = tile / (prm.num_tiles[1] * prm.num_tiles[2]);
    origin[0] = t0 * prm.tile[0];
    origin[1] = t1 * prm.tile[1];
    origin[2] = t2 * prm.tile[2];
}

// Form base node and FP32 weights of point p. Returns false (and raises the
// error flag) when the stencil leaves the ghosted index space.
template <int ORDER>
__device__ __forceinline__ bool point_weights(const TiledParams& prm, int64_t p, int* s, float (*w)[ORDER + 1],
                                              float (*g)[ORDER + 1]) {
    constexpr int nk = ORDER + 1;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double x0 = logical_coord<ORDER>(load_field<double>(prm.points, p, d), prm.mesh.low[d], prm.mesh.rdx[d]);
        float u;
        base_and_offset<ORDER, float>(x0, s[d], u);
        ok &= (x0 >= 0.0) && (s[d] >= 0) && (s[d] + nk <= prm.mesh.ext[d]);
        SplineKernel<ORDER, float>::weights(u, prm.mesh.rdx_f[d], w[d], g[d]);
    }
    if (!ok) raise_error(prm.error_flag, CGX_ERR_OUT_OF_BOUNDS);
    return ok;
}

// Adds v to dof `dof` of node (s + (i,j,k)) of array slot `a`: into the
// shared box when the stencil is inside it, else straight to global memory.
struct P2GSink {
    const TiledParams& prm;
    float* smem;
    const int* l;  // local base node inside the box
    const int* s;  // global base node
    bool inbox;

    __device__ __forceinline__ void add(int slot, int i, int j, int k, int dof, float v) const {
        const TiledArray& ta = prm.arrays[slot];
        if (inbox) {
            const int node = ((l[0] + i) * prm.box[1] + (l[1] + j)) * prm.box[2] + (l[2] + k);
            const int e = node * ta.a.dofs + dof;
            float* base = smem + ta.smem_offset;
            comp_add(base + e, base + prm.box_nodes * ta.a.dofs + e, v);
        } else {
            atomic_add_array(ta.a, node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k), dof, v);
        }
    }
};

template <int ORDER>
__global__ void __launch_bounds__(256) p2g_tiled_kernel(const __grid_constant__ TiledParams prm) {
    constexpr int nk = ORDER + 1;
    extern __shared__ float smem[];
    __shared__ int item_idx;
    const int64_t nwork = *prm.work_count;
    while (true) {
        if (threadIdx.x == 0) item_idx = atomicAdd(prm.work_counter, 1);
        __syncthreads();
        const int64_t widx = item_idx;
        if (widx >= nwork) break;
        const WorkItem it = prm.work[widx];
        int origin[3];
        tile_origin(prm, it.tile, origin);
        for (int i = threadIdx.x; i < prm.smem_floats; i += blockDim.x) smem[i] = 0.0f;
        __syncthreads();

        for (int64_t p = it.begin + threadIdx.x; p < it.end; p += blockDim.x) {
            int s[3];
            float w[3][nk], g[3][nk];
            if (!point_weights<ORDER>(prm, p, s, w, g)) continue;
            int l[3];
            bool inbox = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                l[d] = s[d] - origin[d];
                inbox &= (l[d] >= 0) && (l[d] + nk <= prm.box[d]);
            }
            const P2GSink sink{prm, smem, l, s, inbox};
            for (int o = 0; o < prm.n_ops; ++o) {
                const DOp& op = prm.ops[o];
                const float mult = float(op.mult);
                switch (op.kind) {
                    case CGX_SCALAR_VALUE_P2G: {
                        const float pd = load_field<float>(op.x, p, 0) * mult;
#pragma unroll
                        for (int i = 0; i < nk; ++i)
#pragma unroll
                            for (int j = 0; j < nk; ++j) {
                                const float wij = pd * w[0][i] * w[1][j];
#pragma unroll
                                for (int k = 0; k < nk; ++k) sink.add(op.slot, i, j, k, 0, wij * w[2][k]);
                            }
                        break;
                    }
                    case CGX_VECTOR_VALUE_P2G: {
                        float pd[3];
#pragma unroll
                        for (int d = 0; d < 3; ++d) pd[d] = mult * load_field<float>(op.x, p, d);
#pragma unroll
                        for (int i = 0; i < nk; ++i)
#pragma unroll
                            for (int j = 0; j < nk; ++j) {
                                const float wij = w[0][i] * w[1][j];
#pragma unroll
                                for (int k = 0; k < nk; ++k) {
                                    const float wijk = wij * w[2][k];
#pragma unroll
                                    for (int d = 0; d < 3; ++d) sink.add(op.slot, i, j, k, d, pd[d] * wijk);
                                }
                            }
                        break;
                    }
                    case CGX_SCALAR_GRADIENT_P2G: {
                        const float pd = load_field<float>(op.x, p, 0) * mult;
#pragma unroll
                        for (int i = 0; i < nk; ++i)
#pragma unroll
                            for (int j = 0; j < nk; ++j)
#pragma unroll
                                for (int k = 0; k < nk; ++k) {
                                    sink.add(op.slot, i, j, k, 0, pd * g[0][i] * w[1][j] * w[2][k]);
                                    sink.add(op.slot, i, j, k, 1, pd * w[0][i] * g[1][j] * w[2][k]);
                                    sink.add(op.slot, i, j, k, 2, pd * w[0][i] * w[1][j] * g[2][k]);
                                }
                        break;
                    }
                    case CGX_VECTOR_DIVERGENCE_P2G: {
                        float pd[3];
#pragma unroll
                        for (int d = 0; d < 3; ++d) pd[d] = mult * load_field<float>(op.x, p, d);
#pragma unroll
                        for (int i = 0; i < nk; ++i)
#pragma unroll
                            for (int j = 0; j < nk; ++j)
#pragma unroll
                                for (int k = 0; k < nk; ++k)
                                    sink.add(op.slot, i, j, k, 0,
                                             pd[0] * g[0][i] * w[1][j] * w[2][k] + pd[1] * w[0][i] * g[1][j] * w[2][k] +
                                                 pd[2] * w[0][i] * w[1][j] * g[2][k]);
                        break;
                    }
                    case CGX_TENSOR_DIVERGENCE_P2G: {
                        float pd[3][3];
#pragma unroll
                        for (int a = 0; a < 3; ++a)
#pragma unroll
                            for (int b = 0; b < 3; ++b) pd[a][b] = mult * load_field<float>(op.x, p, a * 3 + b);
#pragma unroll
                        for (int i = 0; i < nk; ++i)
#pragma unroll
                            for (int j = 0; j < nk; ++j)
#pragma unroll
                                for (int k = 0; k < nk; ++k) {
                                    const float rg0 = g[0][i] * w[1][j] * w[2][k];
                                    const float rg1 = w[0][i] * g[1][j] * w[2][k];
                                    const float rg2 = w[0][i] * w[1][j] * g[2][k];
#pragma unroll
                                    for (int d0 = 0; d0 < 3; ++d0)
                                        sink.add(op.slot, i, j, k, d0,
                                                 rg0 * pd[d0][0] + rg1 * pd[d0][1] + rg2 * pd[d0][2]);
                                }
                        break;
                    }
                }
            }
        }
        __syncthreads();
        // Flush: one atomic per touched node and dof, (sum + comp) rounded once.
        for (int slot = 0; slot < prm.n_arrays; ++slot) {
            const TiledArray& ta = prm.arrays[slot];
            const int dofs = ta.a.dofs;
            const int count = prm.box_nodes * dofs;
            const float* sum = smem + ta.smem_offset;
            const float* comp = sum + count;
            for (int e = threadIdx.x; e < count; e += blockDim.x) {
                const float v = sum[e] + comp[e];
                if (v == 0.0f) continue;
                const int node = e / dofs, dof = e - node * dofs;
                const int bk = node % prm.box[2];
                const int bj = (node / prm.box[2]) % prm.box[1];
                const int bi = node / (prm.box[1] * prm.box[2]);
                const int gi = origin[0] + bi, gj = origin[1] + bj, gk = origin[2] + bk;
                if (gi >= prm.mesh.ext[0] || gj >= prm.mesh.ext[1] || gk >= prm.mesh.ext[2]) continue;
                atomic_add_array(ta.a, node_index(prm.mesh, gi, gj, gk), dof, v);
            }
        }
        __syncthreads();
    }
}

template <int ORDER>
__global__ void __launch_bounds__(256) g2p_tiled_kernel(const __grid_constant__ TiledParams prm) {
    constexpr int nk = ORDER + 1;
    extern __shared__ float smem[];
    __shared__ int item_idx;
    const int64_t nwork = *prm.work_count;
    while (true) {
        if (threadIdx.x == 0) item_idx = atomicAdd(prm.work_counter, 1);
        __syncthreads();
        const int64_t widx = item_idx;
        if (widx >= nwork) break;
        const WorkItem it = prm.work[widx];
        int origin[3];
        tile_origin(prm, it.tile, origin);
        // Stage the node box of every source array.
        for (int slot = 0; slot < prm.n_arrays; ++slot) {
            const TiledArray& ta = prm.arrays[slot];
            const int dofs = ta.a.dofs;
            const int count = prm.box_nodes * dofs;
            float* dst = smem + ta.smem_offset;
            for (int e = threadIdx.x; e < count; e += blockDim.x) {
                const int node = e / dofs, dof = e - node * dofs;
                const int bk = node % prm.box[2];
                const int bj = (node / prm.box[2]) % prm.box[1];
                const int bi = node / (prm.box[1] * prm.box[2]);
                const int gi = origin[0] + bi, gj = origin[1] + bj, gk = origin[2] + bk;
                float v = 0.0f;
                if (gi < prm.mesh.ext[0] && gj < prm.mesh.ext[1] && gk < prm.mesh.ext[2])
                    v = load_array<float>(ta.a, node_index(prm.mesh, gi, gj, gk), dof);
                dst[e] = v;
            }
        }
        __syncthreads();

        for (int64_t p = it.begin + threadIdx.x; p < it.end; p += blockDim.x) {
            int s[3];
            float w[3][nk], g[3][nk];
            if (!point_weights<ORDER>(prm, p, s, w, g)) continue;
            int l[3];
            bool inbox = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                l[d] = s[d] - origin[d];
                inbox &= (l[d] >= 0) && (l[d] + nk <= prm.box[d]);
            }
            for (int o = 0; o < prm.n_ops; ++o) {
                const DOp& op = prm.ops[o];
                const TiledArray& ta = prm.arrays[op.slot];
                const int dofs = ta.a.dofs;
                const float* box = smem + ta.smem_offset;
                auto val = [&](int i, int j, int k, int dof) -> float {
                    if (inbox) {
                        const int node = ((l[0] + i) * prm.box[1] + (l[1] + j)) * prm.box[2] + (l[2] + k);
                        return box[node * dofs + dof];
                    }
                    return load_array<float>(ta.a, node_index(prm.mesh, s[0] + i, s[1] + j, s[2] + k), dof);
                };
                const float mult = float(op.mult);
                switch (op.kind) {
                    case CGX_SCALAR_VALUE_G2P: {
                        float r = 0.0f;
#pragma unroll
                        for (int i = 0; i < nk; ++i)
#pragma unroll
                            for (int j = 0; j < nk; ++j)
#pragma unroll
                                for (int k = 0; k < nk; ++k) r += val(i, j, k, 0) * w[0][i] * w[1][j] * w[2][k];
                        add_field<float>(op.x, p, 0, mult * r);
                        break;
                    }
                    case CGX_VECTOR_VALUE_G2P: {
                        float r[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
                        for (int i = 0; i < nk; ++i)
#pragma unroll
                            for (int j = 0; j < nk; ++j) {
                                const float wij = w[0][i] * w[1][j];
#pragma unroll
                                for (int k = 0; k < nk; ++k) {
                                    const float wijk = wij * w[2][k];
#pragma unroll
                                    for (int d = 0; d < 3; ++d) r[d] += val(i, j, k, d) * wijk;
                                }
                            }
#pragma unroll
                        for (int d = 0; d < 3; ++d) add_field<float>(op.x, p, d, mult * r[d]);
                        break;
                    }
                    case CGX_SCALAR_GRADIENT_G2P: {
                        float r[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
                        for (int i = 0; i < nk; ++i)
#pragma unroll
                            for (int j = 0; j < nk; ++j)
#pragma unroll
                                for (int k = 0; k < nk; ++k) {
                                    const float f = val(i, j, k, 0);
                                    r[0] += f * g[0][i] * w[1][j] * w[2][k];
                                    r[1] += f * w[0][i] * g[1][j] * w[2][k];
                                    r[2] += f * w[0][i] * w[1][j] * g[2][k];
                                }
#pragma unroll
                        for (int d = 0; d < 3; ++d) add_field<float>(op.x, p, d, mult * r[d]);
                        break;
                    }
                    case CGX_VECTOR_GRADIENT_G2P: {
                        float r[3][3];
#pragma unroll
                        for (int a = 0; a < 3; ++a)
#pragma unroll
                            for (int b = 0; b < 3; ++b) r[a][b] = 0.0f;
#pragma unroll
                        for (int i = 0; i < nk; ++i)
#pragma unroll
                            for (int j = 0; j < nk; ++j)
#pragma unroll
                                for (int k = 0; k < nk; ++k) {
                                    const float rg[3] = {g[0][i] * w[1][j] * w[2][k], w[0][i] * g[1][j] * w[2][k],
                                                         w[0][i] * w[1][j] * g[2][k]};
                                    float v[3];
#pragma unroll
                                    for (int d = 0; d < 3; ++d) v[d] = val(i, j, k, d);
#pragma unroll
                                    for (int a = 0; a < 3; ++a)
#pragma unroll
                                        for (int b = 0; b < 3; ++b) r[a][b] += rg[a] * v[b];
                                }
#pragma unroll
                        for (int a = 0; a < 3; ++a)
#pragma unroll
                            for (int b = 0; b < 3; ++b) add_field<float>(op.x, p, a * 3 + b, mult * r[a][b]);
                        break;
                    }
                    case CGX_VECTOR_DIVERGENCE_G2P: {
                        float r = 0.0f;
#pragma unroll
                        for (int i = 0; i < nk; ++i)
#pragma unroll
                            for (int j = 0; j < nk; ++j)
#pragma unroll
                                for (int k = 0; k < nk; ++k)
                                    r += val(i, j, k, 0) * g[0][i] * w[1][j] * w[2][k] +
                                         val(i, j, k, 1) * w[0][i] * g[1][j] * w[2][k] +
                                         val(i, j, k, 2) * w[0][i] * w[1][j] * g[2][k];
                        add_field<float>(op.x, p, 0, r * mult);
                        break;
                    }
                }
            }
        }
        __syncthreads();
    }
}

template <int ORDER>
cudaError_t launch_tiled_order(const TiledParams& prm, bool p2g, int sms, size_t smem, cudaStream_t st) {
    const void* fn = p2g ? reinterpret_cast<const void*>(&p2g_tiled_kernel<ORDER>)
                         : reinterpret_cast<const void*>(&g2p_tiled_kernel<ORDER>);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int blocks = sms * per_sm;
    if (p2g)
        p2g_tiled_kernel<ORDER><<<blocks, 256, smem, st>>>(prm);
    else
        g2p_tiled_kernel<ORDER><<<blocks, 256, smem, st>>>(prm);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tiled(const TiledParams& prm, int order, bool p2g, int sms, size_t smem, cudaStream_t st) {
    switch (order) {
        case 1: return launch_tiled_order<1>(prm, p2g, sms, smem, st);
        case 2: return launch_tiled_order<2>(prm, p2g, sms, smem, st);
        case 3: return launch_tiled_order<3>(prm, p2g, sms, smem, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace cgx
