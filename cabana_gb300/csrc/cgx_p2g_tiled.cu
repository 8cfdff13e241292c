// Tiled point-to-grid for particles in tile-major order (FP32-compensated form).
//
// The work is the reference's P2G::value / gradient / divergence scatter
// (grid/src/Cabana_Grid_Interpolation.hpp:437-747) for several functors at
// once, reorganised for a GPU whose shared-memory atomics serialise when a
// warp's lanes hit one address -- which is exactly what happens when the
// particles of a warp share a cell:
//
//  * A work item is a tile and a contiguous run (<= 16384) of its particles,
//    taken 2048 at a time. A prep pass stages the operator inputs in shared
//    memory with bulk (TMA) and asynchronous copies and forms, once per particle, the
//    stencil base node inside the tile's node box and the FP32 in-cell
//    offsets (integer operations only, fixed_logical). It then lists the runs of
//    particles sharing a base node.
//  * Operators are lowered to channels: one grid dof that receives, per
//    point, a * W (value channel) or b . grad W (gradient channel). Channels
//    are grouped (2 value or 1 gradient channel per group for the quadratic
//    spline) so a lane holds its group's whole stencil (27 nodes x channels)
//    in registers. The CTA's 16 warps pull units of work -- (piece, group)
//    and then (window, group) -- from shared counters.
//  * Runs of six or more particles (two or more for the cubic spline) are
//    cut into pieces of <= 1024 particles
//    (a dense cell keeps every warp busy). A piece is walked 32 particles at
//    a time, one particle per lane, each lane adding its particle into its registers; at the end of
//    the piece the warp reduces the registers across lanes with a
//    transpose-reduction (each lane ends with 1/32 of the sums) and adds them
//    into the box with compensated shared atomics -- one shared atomic per
//    node and channel per piece instead of one per particle.
//  * The particles of shorter runs (and stencils outside the box) are
//    compacted into a list, taken 32 at a time and added directly, each lane
//    walking its stencil from a different node so lanes do not collide;
//    outside the box they go to global memory with bounds checks, so the tile
//    ordering never changes the result.
//  * At the end of a work item the box is flushed to the Array, one atomic
//    per touched node and dof, sum and compensation rounded once.
#include "cgx_kernels.cuh"

namespace cgx {

namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kChunk = 2048;        // particles staged in shared memory at a time
// Particles per work item (the host builds items of this size). An item is
// processed in chunks of kChunk with one node box flush at its end, so dense
// tiles flush once per kItem particles.
constexpr int kItem = 16384;
constexpr int kMaxRunWindows = 32;  // register sums cover at most 32 windows per lane
// Runs shorter than small_run<ORDER>() add each particle directly: a warp
// reduction costs about as much as adding a few particles one by one, and a
// short run leaves most of a window's lanes idle. A direct particle costs one
// shared atomic per stencil node and channel, so the threshold falls with the
// stencil size: 6 for linear and quadratic, 2 (single particles) for cubic,
// where 64-node direct adds made a uniform 2^24-particle P2G 27 % slower at 8.
// Quadratic, clumped 2^27 particles / 2^24 uniform + clump, P2G (+ G2P) ms:
// threshold 4: 9.50 / 7.43, 6: 9.54 / 7.04, 8: 9.62 / 7.26, 12: 9.99 / 9.44.
constexpr int kMinSmallRun = 2;
template <int ORDER>
__host__ __device__ constexpr int small_run() { return ORDER >= 3 ? 2 : 6; }
// Long runs are cut into pieces of equal length, at most kPiece particles, so
// that all the warps of a channel group share a dense cell, each piece reduced
// on its own.
constexpr int kPiece = 1024;
constexpr int kMaxPieces = kChunk / kMinSmallRun + kChunk / kPiece + 1;
constexpr int kKeyOutside = -1;     // stencil inside the mesh but outside the box
constexpr int kKeyInvalid = -2;     // stencil outside the ghosted index space

template <int ORDER>
struct P2GShape {
    static constexpr int K = ORDER + 1;
    static constexpr int NODES = K * K * K;
    // Channels per group, sized so a lane's stencil sums fit in <= 128
    // registers (16 warps per SM).
    static constexpr int CV = ORDER >= 3 ? 1 : (ORDER == 2 ? 2 : 4);  // value channels per group
    // Two gradient channels per quadratic group also fit without spills but
    // made the clumped 2^27-particle P2G 10 % slower (10.59 ms against 9.66).
    static constexpr int CG = ORDER >= 2 ? 1 : 3;                     // gradient channels per group
    static constexpr int pad32(int v) { return (v + 31) / 32 * 32; }
    static constexpr int NV = pad32(NODES * CV);
    static constexpr int NG = pad32(NODES * CG);
};

__device__ __forceinline__ void comp_add(float* sum, float* comp, float v) {
    const float old = atomicAdd(sum, v);
    const float s = old + v;
    const float bp = s - old;
    const float e = (old - (s - bp)) + (v - bp);
    if (e != 0.0f) atomicAdd(comp, e);
}

// After the call lane L holds, in v[0 .. N/32), the sums over all lanes of
// the original v[L*N/32 .. (L+1)*N/32).
template <int HALF, int O>
__device__ __forceinline__ void reduce_level(float* v, int lane) {
    const bool upper = (lane & O) != 0;
#pragma unroll
    for (int i = 0; i < HALF; ++i) {
        const float send = upper ? v[i] : v[i + HALF];
        const float keep = upper ? v[i + HALF] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, O);
    }
}

template <int N>
__device__ __forceinline__ void transpose_reduce(float* v, int lane) {
    reduce_level<N / 2, 16>(v, lane);
    reduce_level<N / 4, 8>(v, lane);
    reduce_level<N / 8, 4>(v, lane);
    reduce_level<N / 16, 2>(v, lane);
    reduce_level<N / 32, 1>(v, lane);
}

// Shared-memory offsets of each channel's dof in the node box.
struct ChanSmem {
    int sum_base;  // float offset of (node 0, dof) in the sum half
    int comp_off;  // distance from the sum half to the compensation half
    int dofs;      // node stride
};

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

__device__ __forceinline__ float load_src(const TiledGeom& geo, const Source& src, int64_t p) {
    const DField& f = geo.x[src.op];
    const int64_t o = field_base(f, p) + int64_t(src.comp) * f.comp_stride;
    // raw value: the multiplier is applied where the value is used
    return f.dtype == CGX_F64 ? float(__ldg(reinterpret_cast<const double*>(f.data) + o))
                              : __ldg(reinterpret_cast<const float*>(f.data) + o);
}

__device__ __forceinline__ void prefetch_item(const TiledGeom* g, int n_ops, int64_t b, int64_t e) {
    prefetch_field_range(g->points, b, e);
    for (int o = 0; o < n_ops; ++o) prefetch_field_range(g->x[o], b, e);
}

template <int K>
__device__ __forceinline__ float pick(const float* v, int idx) {
    float r = v[0];
#pragma unroll
    for (int a = 1; a < K; ++a) r = (idx == a) ? v[a] : r;
    return r;
}

// Direct (per-point) contribution of one group: compensated shared atomics
// into the box, or global atomics when the stencil is outside the box. Each
// lane walks its stencil starting at a different node.
template <int ORDER, int TILE, int CH, bool GRAD>
__device__ __forceinline__ void add_direct(const TiledParams& prm, const TiledGeom& geo, float* box_smem, const ChanSmem* cs, int first,
                                           int count, const float (*w)[ORDER + 1], const float (*g)[ORDER + 1],
                                           const float (*coef)[3], bool inbox, int key, const int* s, int lane) {
    constexpr int BB = TILE + ORDER;  // node box extent per dimension
    constexpr int K = ORDER + 1;
    constexpr int NODES = K * K * K;
    // Box offsets of the channels, read once: shared-memory atomics in the
    // loop would otherwise make the compiler reload them at every node.
    int cbase[CH], cdofs[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c) {
        const ChanSmem m = cs[first + (c < count ? c : 0)];
        cbase[c] = m.sum_base + m.comp_off;  // node 0 of the compensation half
        cdofs[c] = m.dofs;
    }
    if (inbox) {
        // Inside the box: the lane starts at layer i = lane % K and walks the
        // K layers cyclically, each layer's K x K (j, k) nodes in a fixed
        // order, with the (j, k) weight products formed once. Lanes of one
        // short run (consecutive lanes, same base node) then start on
        // different layers.
        float ajk[K][K], bjk[K][K], cjk[K][K];
#pragma unroll
        for (int j = 0; j < K; ++j)
#pragma unroll
            for (int k = 0; k < K; ++k) {
                ajk[j][k] = w[1][j] * w[2][k];
                bjk[j][k] = GRAD ? g[1][j] * w[2][k] : 0.0f;
                cjk[j][k] = GRAD ? w[1][j] * g[2][k] : 0.0f;
            }
        int i = lane % K;
#pragma unroll 1
        for (int layer = 0; layer < K; ++layer) {
            const float wi = pick<K>(w[0], i);
            const float gi = GRAD ? pick<K>(g[0], i) : 0.0f;
            const int lbase = key + i * (BB * BB);  // box node of stencil node (i, 0, 0)
#pragma unroll
            for (int j = 0; j < K; ++j)
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const int bnode = lbase + j * BB + k;
#pragma unroll
                    for (int c = 0; c < CH; ++c) {
                        if (c >= count) break;
                        const float v = GRAD ? coef[c][0] * (gi * ajk[j][k]) + coef[c][1] * (wi * bjk[j][k]) +
                                                   coef[c][2] * (wi * cjk[j][k])
                                             : coef[c][0] * (wi * ajk[j][k]);
                        // Direct terms go to the compensation half with a
                        // plain (non-returning) atomic: they are small next to
                        // the run sums held in the sum half, and the flush
                        // adds both.
                        atomicAdd(box_smem + cbase[c] + bnode * cdofs[c], v);
                    }
                }
            i = (i + 1 == K) ? 0 : i + 1;
        }
        return;
    }
    int node = lane % NODES;
#pragma unroll 1
    for (int step = 0; step < NODES; ++step) {
        const int i = node / (K * K), j = (node / K) % K, k = node % K;
        const float wi = pick<K>(w[0], i), wj = pick<K>(w[1], j), wk = pick<K>(w[2], k);
        float wv = 0.0f, g0 = 0.0f, g1 = 0.0f, g2 = 0.0f;
        if (GRAD) {
            const float gi = pick<K>(g[0], i), gj = pick<K>(g[1], j), gk = pick<K>(g[2], k);
            g0 = gi * wj * wk;
            g1 = wi * gj * wk;
            g2 = wi * wj * gk;
        } else {
            wv = wi * wj * wk;
        }
        const int bnode = inbox ? key + (i * BB + j) * BB + k : 0;  // box node of stencil node (i, j, k)
        const int64_t gnode = inbox ? 0 : node_index(geo.mesh, s[0] + i, s[1] + j, s[2] + k);
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            if (c >= count) break;
            const float v = GRAD ? coef[c][0] * g0 + coef[c][1] * g1 + coef[c][2] * g2 : coef[c][0] * wv;
            if (inbox) {
                // Direct terms go to the compensation half with a plain
                // (non-returning) atomic: they are small next to the run
                // sums held in the sum half, and the flush adds both.
                atomicAdd(box_smem + cbase[c] + bnode * cdofs[c], v);
            } else {
                const Channel& ch = prm.channels[first + c];
                atomic_add_array(geo.arr[ch.slot], gnode, ch.dof, v);
            }
        }
        node = (node + 1 == NODES) ? 0 : node + 1;
    }
}

// Register accumulation of this lane's particle (lanes outside the current
// run carry zero coefficients). The coefficients are folded into the
// x-weights first, so each (i, j) pair costs one product per channel (value)
// or three (gradient) before the K fused multiply-adds per node.
template <int ORDER, int CH, bool GRAD>
__device__ __forceinline__ void accumulate(float* acc, const float (*w)[ORDER + 1], const float (*g)[ORDER + 1],
                                           const float (*coef)[3]) {
    constexpr int K = ORDER + 1;
    if (GRAD) {
        // node (i, j, k) += P_ij w_k + Q_ij g_k with
        // P_ij = c0 g_i w_j + c1 w_i g_j and Q_ij = c2 w_i w_j
        float a0[CH][K], a1[CH][K], a2[CH][K];
#pragma unroll
        for (int c = 0; c < CH; ++c)
#pragma unroll
            for (int i = 0; i < K; ++i) {
                a0[c][i] = coef[c][0] * g[0][i];
                a1[c][i] = coef[c][1] * w[0][i];
                a2[c][i] = coef[c][2] * w[0][i];
            }
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = 0; j < K; ++j) {
                float P[CH], Q[CH];
#pragma unroll
                for (int c = 0; c < CH; ++c) {
                    P[c] = fmaf(a0[c][i], w[1][j], a1[c][i] * g[1][j]);
                    Q[c] = a2[c][i] * w[1][j];
                }
#pragma unroll
                for (int k = 0; k < K; ++k)
#pragma unroll
                    for (int c = 0; c < CH; ++c) {
                        float& a = acc[((i * K + j) * K + k) * CH + c];
                        a = fmaf(P[c], w[2][k], fmaf(Q[c], g[2][k], a));
                    }
            }
    } else {
        // node (i, j, k) += (c0 w_i) w_j w_k
        float a0[CH][K];
#pragma unroll
        for (int c = 0; c < CH; ++c)
#pragma unroll
            for (int i = 0; i < K; ++i) a0[c][i] = coef[c][0] * w[0][i];
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = 0; j < K; ++j) {
                float A[CH];
#pragma unroll
                for (int c = 0; c < CH; ++c) A[c] = a0[c][i] * w[1][j];
#pragma unroll
                for (int k = 0; k < K; ++k)
#pragma unroll
                    for (int c = 0; c < CH; ++c) {
                        float& a = acc[((i * K + j) * K + k) * CH + c];
                        a = fmaf(A[c], w[2][k], a);
                    }
            }
    }
}

// Reduce the warp's register sums and add them to the box.
template <int ORDER, int TILE, int CH, int NPAD>
__device__ __forceinline__ void flush_run(float* acc, int lane, int key, const TiledParams& prm, float* box_smem,
                                          const ChanSmem* cs, int first, int count) {
    constexpr int BB = TILE + ORDER;  // node box extent per dimension
    constexpr int K = ORDER + 1;
    constexpr int NODES = K * K * K;
    constexpr int R = NPAD / 32;
    transpose_reduce<NPAD>(acc, lane);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int idx = lane * R + r;
        const int node = idx / CH;
        const int c = idx - node * CH;
        if (node < NODES && c < count && acc[r] != 0.0f) {
            // stencil node (i, j, k) of base key (l0, l1, l2) sits at box index
            // key + (i * BB + j) * BB + k
            const int i = node / (K * K), j = (node / K) % K, k = node % K;
            const int bnode = key + (i * BB + j) * BB + k;
            const ChanSmem m = cs[first + c];
            const int e = m.sum_base + bnode * m.dofs;
            comp_add(box_smem + e, box_smem + e + m.comp_off, acc[r]);
        }
    }
#pragma unroll
    for (int v = 0; v < NPAD; ++v) acc[v] = 0.0f;
}

// The source rows and multipliers of channel group gi, and the per-lane
// coefficient load: coef[c][n] = source n of channel c of particle i times
// its multiplier; raw source s of item particle i is srcs[src_off[s] + i * src_str[s]].
template <int CH, int NS>
struct GroupCoef {
    int first, count;
    int soff[CH][NS];  // staging offset of each source row (-1: none)
    int sstr[CH][NS];  // its stride between particles
    float smul[CH][NS];
    __device__ __forceinline__ GroupCoef(const TiledParams& prm, int gi, const int* src_off, const int* src_str) {
        const ChannelGroup grp = prm.groups[gi];
        first = grp.first;
        count = grp.count;
#pragma unroll
        for (int c = 0; c < CH; ++c)
#pragma unroll
            for (int n = 0; n < NS; ++n) {
                const int rr = c < count ? prm.channels[first + c].src[n] : -1;
                soff[c][n] = rr >= 0 ? src_off[rr] : -1;
                sstr[c][n] = rr >= 0 ? src_str[rr] : 0;
                smul[c][n] = rr >= 0 ? prm.sources[rr].mult : 0.0f;
            }
    }
    __device__ __forceinline__ void load(const float* srcs, int i, bool active, float (*coef)[3]) const {
#pragma unroll
        for (int c = 0; c < CH; ++c)
#pragma unroll
            for (int n = 0; n < 3; ++n) {
                const int m = n < NS ? n : 0;
                const bool has = n < NS && soff[c][m] >= 0;
                coef[c][n] = (has && active) ? srcs[soff[c][m] + i * sstr[c][m]] * smul[c][m] : 0.0f;
            }
    }
};

// One piece [rb, re) of a big cell run (one base node inside the box) for
// channel group gi: register accumulation, then one reduction and one
// compensated shared atomic per node and channel. prep[i] = (u0, u1, u2,
// key) of item particle i.
template <int ORDER, int TILE, bool GRAD>
__device__ __forceinline__ void run_piece(const TiledParams& prm, const TiledGeom& geo, float* box_smem,
                                          const float4* prep, const float* srcs, const int* src_off,
                                          const int* src_str, int2 piece, const ChanSmem* cs, int gi, int lane) {
    using SH = P2GShape<ORDER>;
    constexpr int K = SH::K;
    constexpr int CH = GRAD ? SH::CG : SH::CV;
    constexpr int NPAD = GRAD ? SH::NG : SH::NV;
    const GroupCoef<CH, GRAD ? 3 : 1> gc(prm, gi, src_off, src_str);
    const int first = gc.first, count = gc.count;
    float acc[NPAD];
#pragma unroll
    for (int v = 0; v < NPAD; ++v) acc[v] = 0.0f;
    {
        const int rb = piece.x, re = piece.y;
        const int key = __float_as_int(prep[rb].w);
        int windows = 0;
        for (int w0 = rb; w0 < re; w0 += 32) {
            const int i = w0 + lane;
            const bool active = i < re;
            float coef[CH][3];
            gc.load(srcs, i, active, coef);
            const float4 pu = active ? prep[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            const float u[3] = {pu.x, pu.y, pu.z};
            float w[3][K], g[3][K];
#pragma unroll
            for (int d = 0; d < 3; ++d) SplineKernel<ORDER, float>::weights(u[d], geo.mesh.rdx_f[d], w[d], g[d]);
            if (windows == kMaxRunWindows) {
                flush_run<ORDER, TILE, CH, NPAD>(acc, lane, key, prm, box_smem, cs, first, count);
                windows = 0;
            }
            ++windows;
            accumulate<ORDER, CH, GRAD>(acc, w, g, coef);
        }
        flush_run<ORDER, TILE, CH, NPAD>(acc, lane, key, prm, box_smem, cs, first, count);
    }
}

// One window of the compacted list of particles added directly (single
// particles of their cell, or stencils outside the box), for channel group
// gi: each lane adds its item particle i (-1: none) on its own.
template <int ORDER, int TILE, bool GRAD>
__device__ __forceinline__ void run_window(const TiledParams& prm, const TiledGeom& geo, float* box_smem,
                                           const float4* prep, const float* srcs, const int* src_off,
                                           const int* src_str, int i, const ChanSmem* cs, int gi,
                                           int64_t item_begin, int lane) {
    using SH = P2GShape<ORDER>;
    constexpr int K = SH::K;
    constexpr int CH = GRAD ? SH::CG : SH::CV;
    const GroupCoef<CH, GRAD ? 3 : 1> gc(prm, gi, src_off, src_str);
    const int first = gc.first, count = gc.count;
    {
        const bool active = i >= 0;
        float coef[CH][3];
        gc.load(srcs, active ? i : 0, active, coef);
        if (!active) return;
        const float4 pu = prep[i];
        const int key = __float_as_int(pu.w);
        const float u[3] = {pu.x, pu.y, pu.z};
        float w[3][K], g[3][K];
#pragma unroll
        for (int d = 0; d < 3; ++d) SplineKernel<ORDER, float>::weights(u[d], geo.mesh.rdx_f[d], w[d], g[d]);
        int s[3] = {0, 0, 0};  // global base node, for a stencil outside the box
        const bool inbox = key >= 0;
        if (!inbox) {
            float uu[3];
            form_point<ORDER>(geo, item_begin + i, s, uu);
        }
        add_direct<ORDER, TILE, CH, GRAD>(prm, geo, box_smem, cs, first, count, w, g, coef, inbox, key, s, lane);
    }
}

template <int ORDER, int TILE, bool BATCHED>
__global__ void __launch_bounds__(kThreads, 1) p2g_tiled_kernel(const __grid_constant__ TiledParams prm) {
    constexpr int BB = TILE + ORDER;  // node box extent per dimension
    using SH = P2GShape<ORDER>;
    constexpr int K = ORDER + 1;
    extern __shared__ __align__(16) float smem[];
    float* box_smem = smem;
    float4* prep = reinterpret_cast<float4*>(smem + ((prm.smem_floats + 3) & ~3));
    float* srcs = reinterpret_cast<float*>(prep + kChunk);
    __shared__ ChanSmem cs[kMaxChannels];
    __shared__ int item_idx;
    __shared__ int runs[kChunk + 1];
    __shared__ int2 pieces[kMaxPieces];
    __shared__ unsigned char run_direct[kChunk];  // per run: its particles are added directly
    __shared__ int16_t dlist[kChunk];             // particles added directly, in order
    __shared__ int n_runs, n_big, n_direct;
    __shared__ int next_run[2 * kMaxGroups];
    __shared__ int warp_sums[kWarps];
    __shared__ TiledGeom sgeo;  // instance of the current work item (batched launches)
    int cur_inst = -1;
    const TiledGeom& geo = BATCHED ? sgeo : prm.geom;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = threadIdx.x; c < prm.n_channels; c += blockDim.x) {
        const Channel ch = prm.channels[c];
        const TiledArray& ta = prm.arrays[ch.slot];
        cs[c].sum_base = ta.smem_offset + ch.dof;
        cs[c].comp_off = (BB * BB * BB) * ta.a.dofs;
        cs[c].dofs = ta.a.dofs;
    }
    // Staging regions of the operator inputs: op o owns op_nsrc[o] * kChunk
    // + kOpSlack floats (16-byte aligned); per chunk, src_off / src_str place
    // source s of item particle i at srcs[src_off[s] + i * src_str[s]].
    __shared__ int op_base[kMaxOps], op_nsrc[kMaxOps];
    // Source s is component src_comp[s] of operator src_op[s]'s field, the
    // src_j[s]-th source of that operator.
    __shared__ int8_t src_op[kMaxSources], src_comp[kMaxSources], src_j[kMaxSources];
    // Per operator of the current instance: its FP32 field when the field is
    // dense (vector length 1, components adjacent and all of them sources),
    // which is staged by one bulk copy per chunk; null otherwise.
    __shared__ const float* op_dense[kMaxOps];
    __shared__ int src_off[kMaxSources], src_str[kMaxSources];
    // Dense field blocks arrive by bulk copies completing one phase of
    // src_bar per chunk; a wait that runs out sets `aborted` for the CTA.
    __shared__ uint64_t src_bar;
    __shared__ int aborted;
    unsigned src_phase = 0u;
    if (threadIdx.x == 0) {
        mbar_init(&src_bar);
        aborted = 0;
        int base = 0;
        for (int o = 0; o < prm.n_ops; ++o) {
            int n = 0;
            for (int s = 0; s < prm.n_sources; ++s) {
                if (prm.sources[s].op != o) continue;
                src_op[s] = int8_t(o);
                src_comp[s] = prm.sources[s].comp;
                src_j[s] = int8_t(n++);
            }
            op_base[o] = base;
            op_nsrc[o] = n;
            base += n > 0 ? n * kChunk + kOpSlack : 0;
        }
    }
    __syncthreads();
    // Fill op_dense for the instance in `geo` (threads < n_ops; the caller
    // synchronises before the next stage).
    auto find_dense = [&]() {
        if (threadIdx.x < prm.n_ops) {
            const int o = threadIdx.x, nsrc = op_nsrc[o];
            const DField f = geo.x[o];
            const bool dense =
                nsrc > 0 && f.log2vl == 0 && f.comp_stride == 1 && f.dtype == CGX_F32 && f.soa_stride == nsrc;
            op_dense[o] = dense ? reinterpret_cast<const float*>(f.data) : nullptr;
        }
    };
    if (!BATCHED) find_dense();  // visible after the first item's barrier
    // Issue the staging of particles [sb, sb + slen) (raw values; multipliers
    // are applied at use), all copies in flight together: one bulk copy per
    // dense field, issued by one thread, from the 16-byte boundary at or below
    // the first element (components are then read with the field's stride);
    // component copies for other fields. Returns whether bulk copies were
    // issued (the same in every thread).
    auto stage = [&](int64_t sb, int slen) -> bool {
        if (threadIdx.x < prm.n_sources) {
            const int s = threadIdx.x, o = src_op[s];
            const float* dense = op_dense[o];
            if (dense) {
                const int shift = int((reinterpret_cast<uintptr_t>(dense + sb * op_nsrc[o]) & 15) >> 2);
                src_off[s] = op_base[o] + shift + src_comp[s];
                src_str[s] = op_nsrc[o];
            } else {
                src_off[s] = op_base[o] + src_j[s] * kChunk;
                src_str[s] = 1;
            }
        }
        bool bulk = false;
        for (int o = 0; o < prm.n_ops; ++o) {
            const int nsrc = op_nsrc[o];
            if (nsrc == 0) continue;
            float* region = srcs + op_base[o];
            const float* dense = op_dense[o];
            if (dense) {
                if (threadIdx.x == 0) {
                    if (!bulk) fence_proxy_async();  // after the barrier that ended the buffer's last reads
                    const float* first = dense + sb * nsrc;
                    const int shift = int((reinterpret_cast<uintptr_t>(first) & 15) >> 2);
                    const unsigned bytes = unsigned((shift + slen * nsrc + 3) >> 2) * 16u;
                    mbar_expect_tx(&src_bar, bytes);
                    bulk_copy_g2s(region, first - shift, bytes, &src_bar);
                }
                bulk = true;
                continue;
            }
            const DField f = geo.x[o];
            for (int s = 0; s < prm.n_sources; ++s) {
                if (src_op[s] != o) continue;
                const Source src = prm.sources[s];
                float* dst = region + src_j[s] * kChunk;
                if (f.log2vl == 0 && f.dtype == CGX_F32) {
                    const float* base =
                        reinterpret_cast<const float*>(f.data) + int64_t(src.comp) * f.comp_stride + sb * f.soa_stride;
                    const int64_t stride = f.soa_stride;
                    for (int i = threadIdx.x; i < slen; i += blockDim.x) cp_async4(dst + i, base + i * stride);
                } else {
                    for (int i = threadIdx.x; i < slen; i += blockDim.x) dst[i] = load_src(geo, src, sb + i);
                }
            }
        }
        if (bulk && threadIdx.x == 0) mbar_arrive(&src_bar);
        return bulk;
    };
    const int ng = prm.n_groups;
    const int64_t nwork = *prm.work_count;
    __shared__ int next_idx;  // the item after the current one (its inputs are prefetched into L2)
    if (threadIdx.x == 0) next_idx = atomicAdd(prm.work_counter, 1);
    while (true) {
        if (threadIdx.x == 0) {
            item_idx = next_idx;
            next_idx = atomicAdd(prm.work_counter, 1);
        }
        for (int i = threadIdx.x * 4; i < prm.smem_floats; i += blockDim.x * 4) {
            if (i + 3 < prm.smem_floats)
                *reinterpret_cast<float4*>(box_smem + i) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            else
                for (int j = i; j < prm.smem_floats; ++j) box_smem[j] = 0.0f;
        }
        __syncthreads();
        const int64_t widx = item_idx;
        if (widx >= nwork) break;
        const WorkItem it = prm.work[widx];
        if (BATCHED && it.instance != cur_inst) {
            // all threads are past the previous item's flush (barrier above)
            const int* src = reinterpret_cast<const int*>(prm.instances + it.instance);
            int* dst = reinterpret_cast<int*>(&sgeo);
            for (int i = threadIdx.x; i < int(sizeof(TiledGeom) / 4); i += blockDim.x) dst[i] = src[i];
            cur_inst = it.instance;
            __syncthreads();
            find_dense();
            __syncthreads();
        }
        int origin[3];
        {
            const int t2 = it.tile % geo.num_tiles[2];
            const int t1 = (it.tile / geo.num_tiles[2]) % geo.num_tiles[1];
            const int t0 = it.tile / (geo.num_tiles[1] * geo.num_tiles[2]);
            origin[0] = t0 * prm.tile[0];
            origin[1] = t1 * prm.tile[1];
            origin[2] = t2 * prm.tile[2];
        }
        // The item is processed in chunks of kChunk particles staged in shared
        // memory; the node box accumulates over all of them and is flushed once.
        for (int64_t cb = it.begin; cb < it.end; cb += kChunk) {
            if (threadIdx.x < 2 * kMaxGroups) next_run[threadIdx.x] = 0;
            if (threadIdx.x == 0) n_big = 0;
            const int len = int(it.end - cb < kChunk ? it.end - cb : kChunk);
            const bool bulk = stage(cb, len);
            if (threadIdx.x == 0) {
                // Pull the next chunk's coordinates and operator inputs (of
                // this item, or the first chunk of the next one) into L2 while
                // this chunk is processed: its prep then waits on L2, not HBM.
                const int64_t nidx = next_idx;
                if (cb + kChunk < it.end) {
                    const int64_t ne = cb + 2 * kChunk < it.end ? cb + 2 * kChunk : it.end;
                    prefetch_item(&geo, prm.n_ops, cb + kChunk, ne);
                } else if (nidx < nwork) {
                    const WorkItem nx = prm.work[nidx];
                    const int64_t ne = nx.begin + kChunk < nx.end ? nx.begin + kChunk : nx.end;
                    prefetch_item(BATCHED ? prm.instances + nx.instance : &prm.geom, prm.n_ops, nx.begin, ne);
                }
            }
            // Prep: base node key in the box and in-cell offsets of particles
            // threadIdx.x + q * kThreads (so a warp's coordinate loads cover
            // adjacent particles; all loaded before any is used). The run scan
            // below then takes each thread's kChunk / kThreads consecutive
            // particles.
            constexpr int PER = kChunk / kThreads;
            int keys[PER];
            int rid[PER];  // run index of each of this thread's particles
            {
                double xs[PER][3];
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const int i = threadIdx.x + q * kThreads;
#pragma unroll
                    for (int d = 0; d < 3; ++d) xs[q][d] = i < len ? load_field<double>(geo.points, cb + i, d) : 0.0;
                }
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const int i = threadIdx.x + q * kThreads;
                    if (i >= len) continue;
                    int key = kKeyInvalid;
                    int s[3];
                    float u[3];
                    if (!form_from<ORDER>(geo, xs[q], s, u)) {
                        raise_error(prm.error_flag, CGX_ERR_OUT_OF_BOUNDS);
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
                if (!mbar_wait(&src_bar, src_phase, kMaxPolls)) {
                    raise_error(prm.error_flag, CGX_ERR_TIMEOUT);
                    aborted = 1;
                }
                src_phase ^= 1u;
            }
            __syncthreads();
            if (aborted) break;  // the same in every thread after the barrier
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int i = threadIdx.x * PER + q;
                keys[q] = i < len ? __float_as_int(prep[i].w) : kKeyInvalid;
            }
            // Run starts: particle i starts a run when its key differs from i-1.
            {
                int flags = 0, nstart = 0;
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const int i = threadIdx.x * PER + q;
                    int prev = kKeyInvalid - 1;
                    if (i > 0) prev = q == 0 ? __float_as_int(prep[i - 1].w) : keys[q - 1];
                    const bool st = i < len && keys[q] != prev;
                    flags |= st ? (1 << q) : 0;
                    nstart += st ? 1 : 0;
                }
                // block exclusive scan of nstart
                int x = nstart;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                if (lane == 31) warp_sums[warp] = x;
                __syncthreads();
                int wp = 0;
                for (int w2 = 0; w2 < warp; ++w2) wp += warp_sums[w2];
                int pos = wp + x - nstart;
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    if (flags & (1 << q)) runs[pos++] = threadIdx.x * PER + q;
                    rid[q] = pos - 1;  // run of particle threadIdx.x * PER + q
                }
                if (threadIdx.x == kThreads - 1) {
                    n_runs = pos;
                    runs[pos] = len;
                }
            }
            __syncthreads();
            // Classify runs: long runs inside the box go to the big list, the
            // particles of the others are added directly, window by window.
            for (int r = threadIdx.x; r < n_runs; r += blockDim.x) {
                const int rb = runs[r], re = runs[r + 1];
                const int key = __float_as_int(prep[rb].w);
                const bool is_big = key >= 0 && re - rb >= small_run<ORDER>();
                if (is_big) {
                    // n_big counts pieces: at most kChunk / kPiece + (number of big runs) <= kMaxPieces
                    // np pieces of equal length (to within one particle), so
                    // no short remainder piece leaves its warp idle early
                    const int len_r = re - rb;
                    const int np = (len_r + kPiece - 1) / kPiece;
                    const int base = atomicAdd(&n_big, np);
                    for (int q = 0; q < np; ++q)
                        pieces[base + q] = make_int2(rb + q * len_r / np, rb + (q + 1) * len_r / np);
                }
                run_direct[r] = (!is_big && key != kKeyInvalid) ? 1 : 0;
            }
            __syncthreads();
            // The particles added directly, compacted into a list (in order)
            // so their windows are full: each thread flags its own particles
            // and a block scan places them.
            {
                int dflags = 0, nd = 0;
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const int i = threadIdx.x * PER + q;
                    const bool d = i < len && run_direct[rid[q]] != 0;
                    dflags |= d ? (1 << q) : 0;
                    nd += d ? 1 : 0;
                }
                int x = nd;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                if (lane == 31) warp_sums[warp] = x;
                __syncthreads();
                int pos = x - nd;
                for (int w2 = 0; w2 < warp; ++w2) pos += warp_sums[w2];
#pragma unroll
                for (int q = 0; q < PER; ++q)
                    if (dflags & (1 << q)) dlist[pos++] = int16_t(threadIdx.x * PER + q);
                if (threadIdx.x == kThreads - 1) n_direct = pos;
            }
            __syncthreads();
            {
                // Units of work are (piece, group) and then (window, group),
                // pulled by any warp from two shared counters: every warp stays
                // busy whatever the mix of value and gradient groups.
                const int nunit = n_big * ng, ndir = n_direct, nwin = (ndir + 31) >> 5;
                while (true) {
                    int u = 0;
                    if (lane == 0) u = atomicAdd(&next_run[0], 1);
                    u = __shfl_sync(0xffffffffu, u, 0);
                    if (u >= nunit) break;
                    const int gi = u % ng;
                    const int2 piece = pieces[u / ng];
                    if (prm.groups[gi].gradient)
                        run_piece<ORDER, TILE, true>(prm, geo, box_smem, prep, srcs, src_off, src_str, piece, cs, gi, lane);
                    else
                        run_piece<ORDER, TILE, false>(prm, geo, box_smem, prep, srcs, src_off, src_str, piece, cs, gi, lane);
                }
                const int wunit = nwin * ng;
                while (true) {
                    int u = 0;
                    if (lane == 0) u = atomicAdd(&next_run[1], 1);
                    u = __shfl_sync(0xffffffffu, u, 0);
                    if (u >= wunit) break;
                    const int gi = u % ng, wi = u / ng;
                    const int k = wi * 32 + lane;
                    const int i = k < ndir ? int(dlist[k]) : -1;  // item particle of this lane, or none
                    if (prm.groups[gi].gradient)
                        run_window<ORDER, TILE, true>(prm, geo, box_smem, prep, srcs, src_off, src_str, i, cs, gi, cb,
                                                      lane);
                    else
                        run_window<ORDER, TILE, false>(prm, geo, box_smem, prep, srcs, src_off, src_str, i, cs, gi, cb,
                                                      lane);
                }
            }
            __syncthreads();
        }
        if (aborted) break;  // a bulk copy never completed: stop (the error flag is set)
        // Flush the box: one atomic per touched node and dof.
        for (int slot = 0; slot < prm.n_arrays; ++slot) {
            const TiledArray& ta = prm.arrays[slot];
            const int dofs = ta.a.dofs;
            const int count = (BB * BB * BB) * dofs;
            const float* sum = box_smem + ta.smem_offset;
            const float* comp = sum + count;
            for (int node = threadIdx.x; node < BB * BB * BB; node += blockDim.x) {
                const int bk = node % BB;
                const int bj = (node / BB) % BB;
                const int bi = node / (BB * BB);
                const int gi = origin[0] + bi, gj = origin[1] + bj, gk = origin[2] + bk;
                if (gi >= geo.mesh.ext[0] || gj >= geo.mesh.ext[1] || gk >= geo.mesh.ext[2]) continue;
                const int64_t gnode = node_index(geo.mesh, gi, gj, gk);
                for (int dof = 0; dof < dofs; ++dof) {
                    const int e = node * dofs + dof;
                    const float v = sum[e] + comp[e];
                    if (v != 0.0f) atomic_add_array(geo.arr[slot], gnode, dof, v);
                }
            }
        }
        __syncthreads();
    }
}

size_t smem_bytes(const TiledParams& prm, size_t box_bytes) {
    return (box_bytes + 15) / 16 * 16 + size_t(kChunk) * sizeof(float4) +
           (size_t(prm.n_sources) * kChunk + size_t(prm.n_ops) * kOpSlack) * sizeof(float);
}

template <int ORDER, bool BATCHED>
const void* kernel_fn() {
    return reinterpret_cast<const void*>(&p2g_tiled_kernel<ORDER, kTiledTile, BATCHED>);
}

const void* pick_fn(int order, bool batched) {
    switch (order) {
        case 1: return batched ? kernel_fn<1, true>() : kernel_fn<1, false>();
        case 2: return batched ? kernel_fn<2, true>() : kernel_fn<2, false>();
        case 3: return batched ? kernel_fn<3, true>() : kernel_fn<3, false>();
    }
    return nullptr;
}

// Raise the kernel's dynamic shared-memory limit and report how many CTAs
// fit on one SM (0: the launch cannot run).
cudaError_t prepare(const void* fn, size_t smem, int* per_sm) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, fn, kThreads, smem);
}

template <int ORDER, bool BATCHED>
cudaError_t launch_kernel(const TiledParams& prm, int blocks, size_t smem, cudaStream_t st) {
    p2g_tiled_kernel<ORDER, kTiledTile, BATCHED><<<blocks, kThreads, smem, st>>>(prm);
    return cudaGetLastError();
}

cudaError_t launch_any(const TiledParams& prm, int order, bool batched, int blocks, size_t smem, cudaStream_t st) {
    switch (order) {
        case 1: return batched ? launch_kernel<1, true>(prm, blocks, smem, st) : launch_kernel<1, false>(prm, blocks, smem, st);
        case 2: return batched ? launch_kernel<2, true>(prm, blocks, smem, st) : launch_kernel<2, false>(prm, blocks, smem, st);
        case 3: return batched ? launch_kernel<3, true>(prm, blocks, smem, st) : launch_kernel<3, false>(prm, blocks, smem, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

int p2g_group_capacity(int order, bool gradient) {
    switch (order) {
        case 1: return gradient ? P2GShape<1>::CG : P2GShape<1>::CV;
        case 2: return gradient ? P2GShape<2>::CG : P2GShape<2>::CV;
        case 3: return gradient ? P2GShape<3>::CG : P2GShape<3>::CV;
    }
    return 0;
}

int64_t p2g_tiled_chunk() { return kItem; }

size_t p2g_tiled_smem(const TiledParams& prm, size_t box_bytes) { return smem_bytes(prm, box_bytes); }

size_t p2g_tiled_smem_limit(int order) {
    // the device's opt-in shared memory per block minus the kernel's static
    // tables (the larger of the single and batched instantiations)
    const void* fns[2] = {pick_fn(order, false), pick_fn(order, true)};
    int dev = 0, optin = 0;
    if (!fns[0] || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return 0;
    size_t stat = 0;
    for (const void* fn : fns) {
        cudaFuncAttributes a;
        if (cudaFuncGetAttributes(&a, fn) != cudaSuccess) return 0;
        stat = a.sharedSizeBytes > stat ? a.sharedSizeBytes : stat;
    }
    return size_t(optin) > stat ? size_t(optin) - stat : 0;
}

cudaError_t launch_p2g_tiled(const TiledParams& prm, int order, int sms, size_t smem, cudaStream_t st) {
    const void* fn = pick_fn(order, false);
    if (!fn) return cudaErrorInvalidValue;
    const size_t bytes = smem_bytes(prm, smem);
    int per_sm = 0;
    cudaError_t e = prepare(fn, bytes, &per_sm);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    return launch_any(prm, order, false, sms * per_sm, bytes, st);
}

cudaError_t prepare_p2g_tiled(const TiledParams& prm, int order, bool batched, size_t box_bytes, int* per_sm) {
    const void* fn = pick_fn(order, batched);
    if (!fn) return cudaErrorInvalidValue;
    return prepare(fn, smem_bytes(prm, box_bytes), per_sm);
}

cudaError_t launch_p2g_tiled_prepared(const TiledParams& prm, int order, bool batched, int blocks, size_t box_bytes,
                                      cudaStream_t st) {
    return launch_any(prm, order, batched, blocks, smem_bytes(prm, box_bytes), st);
}

}  // namespace cgx
