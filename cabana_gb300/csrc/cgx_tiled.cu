// Tiled grid-to-point for particles in tile-major order (FP32 form).
//
// A persistent grid pulls work items (a tile and a contiguous run of its
// particles) from a device counter and handles them in three passes over
// sub-runs of up to 1024 particles, so that global memory is touched only in
// long runs of independent loads and stores:
//   1. load: the coordinates are read and turned into the stencil base node
//      inside the tile's node box and FP32 in-cell offsets (integer
//      operations only, fixed_logical); the current values of the point
//      fields being accumulated are copied into shared memory;
//   2. compute: each thread gathers for one particle from the node box staged
//      in shared memory. All operators that read the array share one pass
//      over the stencil that forms, per dof n, the value sum V_n = sum W v_n
//      and the gradient sums D_mn = sum d_m W v_n in factorised
//      (tensor-product) order; each functor takes its result from them:
//        ScalarValueG2P V_0, VectorValueG2P V_n, ScalarGradientG2P D_m0,
//        VectorGradientG2P D_mn, VectorDivergenceG2P sum_m D_mm
//      (grid/src/Cabana_Grid_Interpolation.hpp:53-364, :938-1182), and adds
//      multiplier * result to the staged field values;
//   3. store: the staged field values are written back.
// A point whose stencil leaves the box reads the Array directly, so the
// ordering never changes the result.
#include "cgx_kernels.cuh"

namespace cgx {

namespace {

constexpr int kThreads = 256;
constexpr int kSub = 1024;          // particles per pass
constexpr int kMaxOutCols = 24;     // staged point-field components per launch
constexpr int kKeyOutside = -1;
constexpr int kKeyInvalid = -2;

int g2p_comps(int kind) {
    switch (kind) {
        case CGX_SCALAR_VALUE_G2P: case CGX_VECTOR_DIVERGENCE_G2P: return 1;
        case CGX_VECTOR_VALUE_G2P: case CGX_SCALAR_GRADIENT_G2P: return 3;
        case CGX_VECTOR_GRADIENT_G2P: case CGX_VECTOR_GRADIENT_T_G2P: return 9;
    }
    return 0;
}

__device__ __forceinline__ int dev_g2p_comps(int kind) {
    return (kind == CGX_VECTOR_GRADIENT_G2P || kind == CGX_VECTOR_GRADIENT_T_G2P) ? 9
           : (kind == CGX_VECTOR_VALUE_G2P || kind == CGX_SCALAR_GRADIENT_G2P) ? 3 : 1;
}

template <int ORDER>
__device__ __forceinline__ bool form_from(const TiledGeom& geo, const double* x, int* s, float* u) {
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int c;
        ok &= fixed_logical(x[d], geo.fx[d], c, u[d]);
        s[d] = c + first_offset(ORDER);
        ok &= (s[d] >= 0) && (s[d] + ORDER + 1 <= geo.mesh.ext[d]);
    }
    return ok;
}

template <int ORDER>
__device__ __forceinline__ bool form_point(const TiledGeom& geo, int64_t p, int* s, float* u) {
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int c;
        ok &= fixed_logical(load_field<double>(geo.points, p, d), geo.fx[d], c, u[d]);
        s[d] = c + first_offset(ORDER);
        ok &= (s[d] >= 0) && (s[d] + ORDER + 1 <= geo.mesh.ext[d]);
    }
    return ok;
}

// Gather sums for one array: V[n] = sum W v_n, D[m][n] = sum d_m W v_n.
// BOXED: the stencil's base node is box node `key`, and stencil node
// (i, j, k) is box node key + (i * BB + j) * BB + k; otherwise the array is
// read at the global nodes s + (i, j, k).
template <int ORDER, int TILE, int NDOF, bool GRAD, bool BOXED>
__device__ __forceinline__ void gather_sums(const TiledGeom& geo, const DArray& arr, const float* box, int key,
                                            const int* s, const float (*w)[ORDER + 1],
                                            const float (*g)[ORDER + 1], float* V, float (*D)[3]) {
    constexpr int BB = TILE + ORDER;  // node box extent per dimension
    constexpr int K = ORDER + 1;
    static_assert(NDOF == 1 || NDOF == 3, "one or three gathered dofs");
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
                    // box nodes are padded to 4 floats for 3 dofs: one 16-byte load per node
                    const int node = key + (i * BB + j) * BB + k;
                    if constexpr (NDOF == 3) {
                        const float4 q = reinterpret_cast<const float4*>(box)[node];
                        v[0] = q.x;
                        v[1 < NDOF ? 1 : 0] = q.y;
                        v[2 < NDOF ? 2 : 0] = q.z;
                    } else {
                        v[0] = box[node];
                    }
                } else {
                    const int64_t node = node_index(geo.mesh, s[0] + i, s[1] + j, s[2] + k);
#pragma unroll
                    for (int n = 0; n < NDOF; ++n) v[n] = load_array<float>(arr, node, n);
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

// Where a pass stages the point-field values of operator o: component c of
// pass particle i is out[base[o] + i * pstr[o] + c * cstr[o]] (base -1: the
// operator reads another array).
struct OutMap {
    int base[kMaxOps];
    int pstr[kMaxOps];
    int cstr[kMaxOps];
};

// Adds multiplier * result of every operator of this launch into the staged
// point-field values.
template <int NDOF>
__device__ __forceinline__ void apply_ops(const TiledParams& prm, const OutMap& om, float* out, int i, const float* V,
                                          const float (*D)[3]) {
    for (int o = 0; o < prm.n_ops; ++o) {
        const int base = om.base[o];
        if (base < 0) continue;
        const DOp& op = prm.ops[o];
        const float mult = op.mult_f;
        float* x = out + base + i * om.pstr[o];
        const int cs = om.cstr[o];
        switch (op.kind) {
            case CGX_SCALAR_VALUE_G2P:
                x[0] += mult * V[0];
                break;
            case CGX_VECTOR_VALUE_G2P:
#pragma unroll
                for (int d = 0; d < 3; ++d) x[d * cs] += mult * V[d < NDOF ? d : 0];
                break;
            case CGX_SCALAR_GRADIENT_G2P:
#pragma unroll
                for (int d = 0; d < 3; ++d) x[d * cs] += mult * D[d][0];
                break;
            case CGX_VECTOR_GRADIENT_G2P:
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b) x[(a * 3 + b) * cs] += mult * D[a][b < NDOF ? b : 0];
                break;
            case CGX_VECTOR_GRADIENT_T_G2P:
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b) x[(b * 3 + a) * cs] += mult * D[a][b < NDOF ? b : 0];
                break;
            case CGX_VECTOR_DIVERGENCE_G2P:
                x[0] += (D[0][0] + D[1][1 < NDOF ? 1 : 0] + D[2][2 < NDOF ? 2 : 0]) * mult;
                break;
        }
    }
}

template <int ORDER, int TILE, int NDOF, bool GRAD, bool BATCHED>
__global__ void __launch_bounds__(kThreads, 2)
    g2p_tiled_kernel(const __grid_constant__ TiledParams prm, int slot) {
    constexpr int BB = TILE + ORDER;  // node box extent per dimension
    constexpr int K = ORDER + 1;
    extern __shared__ __align__(16) float smem[];
    constexpr int BSTR = NDOF == 3 ? 4 : 1;  // floats per box node
    constexpr int box_floats = ((BB * BB * BB) * BSTR + 3) & ~3;
    float* box = smem;
    float4* prep = reinterpret_cast<float4*>(smem + box_floats);
    float* out = reinterpret_cast<float*>(prep + kSub);
    __shared__ int item_idx;
    __shared__ TiledGeom sgeo;  // instance of the current work item (batched launches)
    int cur_inst = -1;
    const TiledGeom& geo = BATCHED ? sgeo : prm.geom;
    const int64_t nwork = *prm.work_count;
    // Staging of the point fields of the operators reading array `slot`:
    // operator o owns ncomp[o] * kSub + kOpSlack floats of `out` from
    // region[o] (16-byte aligned; -1 for operators of other arrays). A dense
    // FP32 field (vector length 1, its components adjacent) is staged in its
    // own layout by one bulk copy per pass and written back by one bulk copy
    // of its 16-byte aligned interior plus plain stores of the ragged ends;
    // other fields are staged one component (kSub floats) at a time.
    __shared__ int region[kMaxOps], ncomp[kMaxOps];
    __shared__ float* dense_of[kMaxOps];  // per instance: the dense field, or null
    __shared__ OutMap om;                 // per pass
    // Bulk loads complete one phase of ld_bar per pass; a wait that runs out
    // sets `aborted` for the CTA.
    __shared__ uint64_t ld_bar;
    __shared__ int aborted;
    unsigned ld_phase = 0u;
    if (threadIdx.x == 0) {
        mbar_init(&ld_bar);
        aborted = 0;
        int base = 0;
        for (int o = 0; o < prm.n_ops; ++o) {
            const bool mine = prm.ops[o].slot == slot;
            const int nc = mine ? dev_g2p_comps(prm.ops[o].kind) : 0;
            region[o] = mine ? base : -1;
            ncomp[o] = nc;
            base += mine ? nc * kSub + kOpSlack : 0;
        }
    }
    __syncthreads();
    // Fill dense_of for the instance in `geo` (threads < n_ops; the caller
    // synchronises before the next pass).
    auto find_dense = [&]() {
        if (threadIdx.x < prm.n_ops) {
            const int o = threadIdx.x, nc = ncomp[o];
            const DField f = geo.x[o];
            const bool dense = region[o] >= 0 && f.log2vl == 0 && f.comp_stride == 1 && f.soa_stride == nc &&
                               f.dtype == CGX_F32;
            dense_of[o] = dense ? reinterpret_cast<float*>(f.data) : nullptr;
        }
    };
    if (!BATCHED) find_dense();  // visible after the first item's barrier
    while (true) {
        if (threadIdx.x == 0) item_idx = atomicAdd(prm.work_counter, 1);
        __syncthreads();
        const int64_t widx = item_idx;
        if (widx >= nwork) break;
        const WorkItem it = prm.work[widx];
        if (BATCHED && it.instance != cur_inst) {
            // every thread finished the previous item (barrier after its last store)
            const int* src = reinterpret_cast<const int*>(prm.instances + it.instance);
            int* dst = reinterpret_cast<int*>(&sgeo);
            for (int i = threadIdx.x; i < int(sizeof(TiledGeom) / 4); i += blockDim.x) dst[i] = src[i];
            cur_inst = it.instance;
            __syncthreads();
            find_dense();
            __syncthreads();
        }
        const DArray& arr = geo.arr[slot];
        int origin[3];
        {
            const int t2 = it.tile % geo.num_tiles[2];
            const int t1 = (it.tile / geo.num_tiles[2]) % geo.num_tiles[1];
            const int t0 = it.tile / (geo.num_tiles[1] * geo.num_tiles[2]);
            origin[0] = t0 * prm.tile[0];
            origin[1] = t1 * prm.tile[1];
            origin[2] = t2 * prm.tile[2];
        }
        // Stage the gathered dofs of the node box (rows of k are contiguous
        // in the array), as asynchronous copies that complete with the first
        // sub-batch's copies; nodes beyond the mesh read as zero.
        {
            const float* adata = reinterpret_cast<const float*>(arr.data);
            for (int node = threadIdx.x; node < BB * BB * BB; node += blockDim.x) {
                const int bk = node % BB;
                const int bj = (node / BB) % BB;
                const int bi = node / (BB * BB);
                const int gi = origin[0] + bi, gj = origin[1] + bj, gk = origin[2] + bk;
                const bool in = gi < geo.mesh.ext[0] && gj < geo.mesh.ext[1] && gk < geo.mesh.ext[2];
                if (in && arr.dtype == CGX_F32) {
                    const int64_t gnode = node_index(geo.mesh, gi, gj, gk);
#pragma unroll
                    for (int dof = 0; dof < NDOF; ++dof) cp_async4(box + node * BSTR + dof, adata + gnode * arr.dofs + dof);
                } else if (in) {  // double arrays are rounded to FP32 on the way
                    const int64_t gnode = node_index(geo.mesh, gi, gj, gk);
#pragma unroll
                    for (int dof = 0; dof < NDOF; ++dof) box[node * BSTR + dof] = load_array<float>(arr, gnode, dof);
                } else {
#pragma unroll
                    for (int dof = 0; dof < NDOF; ++dof) box[node * BSTR + dof] = 0.0f;
                }
            }
        }
        for (int64_t sb = it.begin; sb < it.end; sb += kSub) {
            const int len = int((it.end - sb < kSub) ? it.end - sb : kSub);
            // 1. load. Current point-field values first (bulk copies of dense
            // fields, asynchronous copies of single components otherwise),
            // then the coordinates, all of a thread's particles loaded
            // before any is used.
            if (threadIdx.x < prm.n_ops) {
                const int o = threadIdx.x;
                const float* d = dense_of[o];
                if (region[o] < 0) {
                    om.base[o] = -1;
                } else if (d) {
                    const int shift = int((reinterpret_cast<uintptr_t>(d + sb * ncomp[o]) >> 2) & 3);
                    om.base[o] = region[o] + shift;
                    om.pstr[o] = ncomp[o];
                    om.cstr[o] = 1;
                } else {
                    om.base[o] = region[o];
                    om.pstr[o] = 1;
                    om.cstr[o] = kSub;
                }
            }
            bool bulk = false;  // the same in every thread
            for (int o = 0; o < prm.n_ops; ++o) {
                if (region[o] < 0) continue;
                const int nc = ncomp[o];
                const float* d = dense_of[o];
                if (d) {
                    if (threadIdx.x == 0) {
                        if (!bulk) {
                            bulk_wait_read();     // the previous pass's write-back has read the region
                            fence_proxy_async();  // after the barrier that ended the region's last accesses
                        }
                        const float* first = d + sb * nc;
                        const int shift = int((reinterpret_cast<uintptr_t>(first) >> 2) & 3);
                        const unsigned bytes = unsigned((shift + len * nc + 3) >> 2) * 16u;
                        mbar_expect_tx(&ld_bar, bytes);
                        bulk_copy_g2s(out + region[o], first - shift, bytes, &ld_bar);
                    }
                    bulk = true;
                    continue;
                }
                const DField& fx = geo.x[o];
                for (int c = 0; c < nc; ++c) {
                    float* dst = out + region[o] + c * kSub;
                    if (fx.log2vl == 0) {
                        const float* src =
                            reinterpret_cast<const float*>(fx.data) + int64_t(c) * fx.comp_stride + sb * fx.soa_stride;
                        const int64_t stride = fx.soa_stride;
                        for (int i = threadIdx.x; i < len; i += blockDim.x) cp_async4(dst + i, src + i * stride);
                    } else {
                        for (int i = threadIdx.x; i < len; i += blockDim.x) dst[i] = load_field<float>(fx, sb + i, c);
                    }
                }
            }
            if (bulk && threadIdx.x == 0) mbar_arrive(&ld_bar);
            {
                constexpr int PER = kSub / kThreads;
                double xs[PER][3];
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const int i = threadIdx.x + q * kThreads;
#pragma unroll
                    for (int d = 0; d < 3; ++d) xs[q][d] = i < len ? load_field<double>(geo.points, sb + i, d) : 0.0;
                }
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const int i = threadIdx.x + q * kThreads;
                    if (i >= len) continue;
                    int s[3];
                    float u[3];
                    int key;
                    if (!form_from<ORDER>(geo, xs[q], s, u)) {
                        raise_error(prm.error_flag, CGX_ERR_OUT_OF_BOUNDS);
                        key = kKeyInvalid;
                    } else {
                        int l[3];
                        bool inbox = true;
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            l[d] = s[d] - origin[d];
                            inbox &= (l[d] >= 0) && (l[d] + K <= BB);
                        }
                        key = inbox ? (l[0] * BB + l[1]) * BB + l[2] : kKeyOutside;
                    }
                    prep[i] = make_float4(u[0], u[1], u[2], __int_as_float(key));
                }
            }
            cp_async_wait_all();
            if (bulk) {
                if (!mbar_wait(&ld_bar, ld_phase, kMaxPolls)) {
                    raise_error(prm.error_flag, CGX_ERR_TIMEOUT);
                    aborted = 1;
                }
                ld_phase ^= 1u;
            }
            __syncthreads();
            if (aborted) break;  // the same in every thread after the barrier
            // 2. compute
            for (int i = threadIdx.x; i < len; i += blockDim.x) {
                const float4 pu = prep[i];
                const int key = __float_as_int(pu.w);
                if (key == kKeyInvalid) continue;
                const float u[3] = {pu.x, pu.y, pu.z};
                float w[3][K], g[3][K];
#pragma unroll
                for (int d = 0; d < 3; ++d) SplineKernel<ORDER, float>::weights(u[d], geo.mesh.rdx_f[d], w[d], g[d]);
                float V[NDOF], D[3][3];
                int s[3];
                if (key >= 0) {
                    gather_sums<ORDER, TILE, NDOF, GRAD, true>(geo, arr, box, key, s, w, g, V, D);
                } else {
                    float uu[3];
                    form_point<ORDER>(geo, sb + i, s, uu);
                    gather_sums<ORDER, TILE, NDOF, GRAD, false>(geo, arr, box, 0, s, w, g, V, D);
                }
                apply_ops<NDOF>(prm, om, out, i, V, D);
            }
            fence_proxy_async();  // the staged values are read by bulk copies below
            __syncthreads();
            // 3. store
            for (int o = 0; o < prm.n_ops; ++o) {
                if (region[o] < 0) continue;
                const int nc = ncomp[o];
                float* d = dense_of[o];
                if (d) {
                    // elements [0, n) of the pass start at `first` and at
                    // out[base]; [head, head + body) is 16-byte aligned at both
                    float* first = d + sb * nc;
                    const int base = om.base[o], n = len * nc;
                    const int head = min(n, int((4 - ((reinterpret_cast<uintptr_t>(first) >> 2) & 3)) & 3));
                    const int body = (n - head) & ~3;
                    if (threadIdx.x == 0 && body > 0)
                        bulk_copy_s2g(first + head, out + base + head, unsigned(body) * 4u);
                    const int t = threadIdx.x;
                    if (t < head) {
                        first[t] = out[base + t];
                    } else if (t >= 4 && t < 4 + (n - head - body)) {
                        const int e = head + body + (t - 4);
                        first[e] = out[base + e];
                    }
                    continue;
                }
                const DField& fx = geo.x[o];
                for (int c = 0; c < nc; ++c) {
                    const float* srcv = out + region[o] + c * kSub;
                    if (fx.log2vl == 0) {
                        float* dst = reinterpret_cast<float*>(fx.data) + int64_t(c) * fx.comp_stride + sb * fx.soa_stride;
                        const int64_t stride = fx.soa_stride;
                        for (int i = threadIdx.x; i < len; i += blockDim.x) dst[i * stride] = srcv[i];
                    } else {
                        float* data = reinterpret_cast<float*>(fx.data);
                        for (int i = threadIdx.x; i < len; i += blockDim.x) data[field_offset(fx, sb + i, c)] = srcv[i];
                    }
                }
            }
            if (threadIdx.x == 0) bulk_commit();
            __syncthreads();
        }
        if (aborted) break;  // a bulk copy never completed: stop (the error flag is set)
    }
    if (threadIdx.x == 0) bulk_wait_all();  // write-backs complete before the CTA exits
}

// launch == false: raise the shared-memory limit and report the resident
// CTAs per SM in *per_sm; launch == true: launch `blocks` CTAs.
template <int ORDER, int NDOF, bool GRAD, bool BATCHED>
cudaError_t g2p_op(const TiledParams& prm, int slot, bool launch, int blocks, size_t smem, cudaStream_t st,
                   int* per_sm) {
    if (!launch) {
        const void* fn = reinterpret_cast<const void*>(&g2p_tiled_kernel<ORDER, kTiledTile, NDOF, GRAD, BATCHED>);
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, fn, kThreads, smem);
    }
    g2p_tiled_kernel<ORDER, kTiledTile, NDOF, GRAD, BATCHED><<<blocks, kThreads, smem, st>>>(prm, slot);
    return cudaGetLastError();
}

template <int ORDER, bool BATCHED>
cudaError_t g2p_shape(const TiledParams& prm, int slot, int ndof, bool grad, bool launch, int blocks, size_t smem,
                      cudaStream_t st, int* per_sm) {
    if (ndof == 3)
        return grad ? g2p_op<ORDER, 3, true, BATCHED>(prm, slot, launch, blocks, smem, st, per_sm)
                    : g2p_op<ORDER, 3, false, BATCHED>(prm, slot, launch, blocks, smem, st, per_sm);
    return grad ? g2p_op<ORDER, 1, true, BATCHED>(prm, slot, launch, blocks, smem, st, per_sm)
                : g2p_op<ORDER, 1, false, BATCHED>(prm, slot, launch, blocks, smem, st, per_sm);
}

cudaError_t g2p_any(const TiledParams& prm, int order, int slot, bool batched, bool launch, int blocks, size_t smem,
                    cudaStream_t st, int* per_sm) {
    int ndof;
    bool grad;
    g2p_slot_need(prm, slot, ndof, grad);
    switch (order) {
        case 1: return batched ? g2p_shape<1, true>(prm, slot, ndof, grad, launch, blocks, smem, st, per_sm)
                               : g2p_shape<1, false>(prm, slot, ndof, grad, launch, blocks, smem, st, per_sm);
        case 2: return batched ? g2p_shape<2, true>(prm, slot, ndof, grad, launch, blocks, smem, st, per_sm)
                               : g2p_shape<2, false>(prm, slot, ndof, grad, launch, blocks, smem, st, per_sm);
        case 3: return batched ? g2p_shape<3, true>(prm, slot, ndof, grad, launch, blocks, smem, st, per_sm)
                               : g2p_shape<3, false>(prm, slot, ndof, grad, launch, blocks, smem, st, per_sm);
    }
    return cudaErrorInvalidValue;
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
            case CGX_VECTOR_GRADIENT_T_G2P:
            case CGX_VECTOR_DIVERGENCE_G2P: ndof = 3; grad = true; break;
        }
    }
}

size_t g2p_tiled_smem(const TiledParams& prm, int slot) {
    int cols = 0;
    bool f64_out = false;
    for (int o = 0; o < prm.n_ops; ++o)
        if (prm.ops[o].slot == slot) {
            cols += g2p_comps(prm.ops[o].kind);
            f64_out |= prm.ops[o].x.dtype == CGX_F64;
        }
    // Point fields are staged as FP32: double fields, or too many components,
    // are left to the point-parallel kernel.
    if (cols > kMaxOutCols || f64_out) return size_t(1) << 30;
    int ndof;
    bool grad;
    g2p_slot_need(prm, slot, ndof, grad);
    const size_t box = size_t((prm.box_nodes * (ndof == 3 ? 4 : 1) + 3) & ~3) * sizeof(float);
    int n_slot_ops = 0;
    for (int o = 0; o < prm.n_ops; ++o) n_slot_ops += prm.ops[o].slot == slot ? 1 : 0;
    return box + size_t(kSub) * sizeof(float4) + (size_t(cols) * kSub + size_t(n_slot_ops) * kOpSlack) * sizeof(float);
}

cudaError_t launch_g2p_tiled(const TiledParams& prm, int order, int slot, int sms, size_t smem, cudaStream_t st) {
    int per_sm = 0;
    cudaError_t e = g2p_any(prm, order, slot, false, false, 0, smem, st, &per_sm);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    return g2p_any(prm, order, slot, false, true, sms * per_sm, smem, st, nullptr);
}

cudaError_t prepare_g2p_tiled(const TiledParams& prm, int order, int slot, bool batched, size_t smem, int* per_sm) {
    return g2p_any(prm, order, slot, batched, false, 0, smem, nullptr, per_sm);
}

cudaError_t launch_g2p_tiled_prepared(const TiledParams& prm, int order, int slot, bool batched, int blocks,
                                      size_t smem, cudaStream_t st) {
    return g2p_any(prm, order, slot, batched, true, blocks, smem, st, nullptr);
}

}  // namespace cgx
