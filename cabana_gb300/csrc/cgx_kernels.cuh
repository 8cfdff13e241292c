// Kernel parameter blocks and launcher entry points (host <-> .cu files).
#pragma once

#include "cgx_internal.cuh"

namespace cgx {

struct PointParams {
    DMesh mesh;
    DField points;
    int64_t num_point;
    int32_t n_ops;
    int32_t dims;  // 3, or 2 for a 2D mesh (mesh.ext[2] == 1; points hold 2 coordinates)
    int32_t n_g2p;  // fused g2p2g: ops[0, n_g2p) are G2P, the rest P2G
    int32_t reserved;
    int* error_flag;
    DOp ops[kMaxOps];
};

struct HaloParams {
    char* data;
    int32_t dtype;
    int32_t dofs;
    int32_t ext[3];
    int32_t owned_cells[3];
    int32_t periodic[3];
    int32_t halo_width;
    int32_t node_extra;  // 1 for nodes, 0 for cells
    int32_t dims;        // 3, or 2 (the single k layer of a 2D array is owned)
    int32_t reserved;
};

// One distinct grid array touched by a tiled launch.
struct TiledArray {
    DArray a;
    int32_t smem_offset;  // float offset of this array's node box in shared memory
    int32_t reserved;
};

// A unit of tiled work: particles [begin, end) of the tile-major order of
// instance `instance` (0 for a single launch), all filed under tile `tile`.
struct WorkItem {
    int64_t begin;
    int64_t end;
    int32_t tile;
    int32_t instance;
};

// One accumulation channel of a tiled p2g launch: a dof of a target array
// that receives, per point, either a * W (value channel) or b . grad W
// (gradient channel). src[] index the source table; -1 means zero.
struct Channel {
    int8_t slot;
    int8_t dof;
    int8_t src[3];
    int8_t reserved[3];
};

// A per-point input value of a tiled p2g launch: component `comp` of the
// field of operator `op`, times the operator's multiplier.
struct Source {
    int8_t op;
    int8_t comp;
    int16_t reserved;
    float mult;
};

constexpr int kMaxSources = 16;

// A set of channels processed together by one warp role.
struct ChannelGroup {
    int8_t gradient;  // 0: value channels, 1: gradient channels
    int8_t first;
    int8_t count;
    int8_t reserved;
};

// Cubic tile edge (base nodes) of the tiled kernels; the node box of a tile
// is kTiledTile + order nodes per dimension, a compile-time constant.
constexpr int kTiledTile = 8;

constexpr int kMaxChannels = 24;
constexpr int kMaxGroups = 16;

// The mesh and buffers of one instance of a tiled launch. A single launch
// carries one in TiledParams::geom; a batched launch (many independent
// meshes of the same operator structure) reads one per work item from
// TiledParams::instances.
struct TiledGeom {
    DMesh mesh;
    double c0[3];  // -low * rdx + (0.5 for even orders): t = x * rdx + c0
    FixedMap fx[3];  // the same mapping in integer form (fixed_logical)
    int32_t num_tiles[3];
    int32_t reserved;
    DField points;
    DField x[kMaxOps];    // point field of operator o
    DArray arr[kMaxOps];  // distinct grid array `slot`
};

struct TiledParams {
    TiledGeom geom;
    const TiledGeom* instances;  // device; null for a single instance
    int64_t num_point;
    int32_t n_ops;
    int32_t n_arrays;
    int32_t tile[3];
    int32_t box[3];        // node box per tile: tile + num_knot - 1
    int32_t box_nodes;     // box[0] * box[1] * box[2]
    int32_t smem_floats;   // floats of shared memory used for node boxes
    int32_t reserved;
    const WorkItem* work;
    const int64_t* work_count;  // device: number of work items
    int* work_counter;          // device: dynamic scheduler counter (zeroed per launch)
    int* error_flag;
    DOp ops[kMaxOps];
    TiledArray arrays[kMaxOps];
    int32_t n_channels;
    int32_t n_groups;
    int32_t n_sources;
    int32_t reserved2;
    Channel channels[kMaxChannels];
    ChannelGroup groups[kMaxGroups];
    Source sources[kMaxSources];
};

// One term of the position adjoint: per point,
//   dL/dx_e += mult * sum_n ( r_n dW_n/dx_e + sum_d q_n[d] d2W_n/(dx_e dx_d) )
// where r_n and q_n pair the point field `s` with the dofs A of array `a` at
// node n according to `pattern`.
enum AdjointPattern : int32_t {
    kAdjValue1 = 0,   // r = s A0                       (ScalarValue P2G / G2P)
    kAdjValue3 = 1,   // r = sum_c s_c A_c              (VectorValue P2G / G2P)
    kAdjGradA = 2,    // q_d = s A_d                    (ScalarGradientP2G, VectorDivergenceG2P)
    kAdjGradS = 3,    // q_d = s_d A0                   (VectorDivergenceP2G, ScalarGradientG2P)
    kAdjTensor = 4,   // q_b = sum_a s[a][b] A_a        (TensorDivergenceP2G, transposed VectorGradientG2P)
    kAdjTensorT = 5,  // q_a = sum_b s[a][b] A_b        (transposed TensorDivergenceP2G, VectorGradientG2P)
};

struct AdjointTerm {
    int32_t pattern;
    float mult_f;
    double mult;
    DField s;
    DArray a;
};

struct AdjointParams {
    DMesh mesh;
    DField points;
    DField points_bar;
    int64_t num_point;
    int32_t n_terms;
    int32_t reserved;
    int* error_flag;
    AdjointTerm terms[kMaxOps];
};

// Message returned by cgx_last_error() on this thread.
void set_last_error(const char* msg);

// Halo modes on one rank. Gather / scatter-sum are Halo::gather and
// Halo::scatter(Sum); the other two are their adjoints (exact transposes).
enum HaloMode : int {
    kHaloGather = 0,        // ghost = owned image
    kHaloScatterSum = 1,    // owned image += ghost
    kHaloGatherAdd = 2,     // ghost += owned image        (adjoint of scatter-sum)
    kHaloScatterClear = 3,  // owned image += ghost; ghost = 0   (adjoint of gather)
};

cudaError_t launch_points(const PointParams& prm, int order, bool p2g, bool fp64, int sms, cudaStream_t st);
// Fused g2p2g on the point kernels (3D): ops[0, prm.n_g2p) G2P, then P2G.
cudaError_t launch_g2p2g_points(const PointParams& prm, int order, bool fp64, int sms, cudaStream_t st);
cudaError_t launch_adjoint_points(const AdjointParams& prm, int order, bool fp64, int sms, cudaStream_t st);
// dL/dx_e += mult * sum_c s_c D[e][c] from the gradient sums D of a value
// term (grads: per point 3 x ncomp floats, ncomp 1 or 3).
cudaError_t launch_adjoint_value_combine(const DField& points_bar, const DField& sf, const float* grads, int64_t n,
                                         int ncomp, float mult, int sms, cudaStream_t st);
cudaError_t launch_halo(const HaloParams& h, int mode, int sms, cudaStream_t st);
cudaError_t launch_fill(void* data, int dtype, int64_t count, double value, int sms, cudaStream_t st);

// Tiled g2p for the operators reading array `slot` (its node box is staged at
// shared offset 0).
cudaError_t launch_g2p_tiled(const TiledParams& prm, int order, int slot, int sms, size_t smem_bytes, cudaStream_t st);
cudaError_t launch_p2g_tiled(const TiledParams& prm, int order, int sms, size_t smem_bytes, cudaStream_t st);
// Two-step form of the tiled launches for plans that are launched many
// times (and may be captured into a CUDA graph): prepare once (sets the
// kernel's shared-memory limit, reports resident CTAs per SM), then launch
// with an explicit CTA count. `batched` selects the kernels that read
// TiledParams::instances. For p2g, `smem_bytes` is the node-box bytes as in
// p2g_tiled_smem; for g2p it is the full dynamic shared memory.
cudaError_t prepare_p2g_tiled(const TiledParams& prm, int order, bool batched, size_t box_bytes, int* per_sm);
cudaError_t launch_p2g_tiled_prepared(const TiledParams& prm, int order, bool batched, int blocks, size_t box_bytes,
                                      cudaStream_t st);
cudaError_t prepare_g2p_tiled(const TiledParams& prm, int order, int slot, bool batched, size_t smem, int* per_sm);
cudaError_t launch_g2p_tiled_prepared(const TiledParams& prm, int order, int slot, bool batched, int blocks,
                                      size_t smem, cudaStream_t st);
// Dofs gathered (1 or 3) and whether gradient sums are needed for array `slot`.
void g2p_slot_need(const TiledParams& prm, int slot, int& ndof, bool& grad);
// Channels per group of the tiled p2g kernel for a spline order.
int p2g_group_capacity(int order, bool gradient);
// Dynamic shared memory of the tiled g2p kernel for array `slot` (huge when
// the launch cannot be tiled: double point fields or too many components).
size_t g2p_tiled_smem(const TiledParams& prm, int slot);
// Particles per work item of the tiled kernels.
int64_t p2g_tiled_chunk();
// Largest dynamic shared memory the tiled p2g kernel of a spline order can
// be launched with on the current device (0 if it cannot be queried).
size_t p2g_tiled_smem_limit(int order);
// Dynamic shared memory of the tiled p2g kernel: node boxes + per-item
// staging of base keys, offsets and sources.
size_t p2g_tiled_smem(const TiledParams& prm, size_t box_bytes);

// Sorting / binning (cgx_sort.cu). Scratch comes from the caller.
size_t radix_sort_scratch_bytes(int64_t n);
// Stable sort of (keys, index) by key. keys_in is consumed (may be
// overwritten). The sorted original indices land in perm_out (uint64).
cudaError_t radix_sort_pairs(uint32_t* keys_in, int64_t n, int key_bits, uint64_t* perm_out, const uint64_t* vals_in,
                             uint64_t val_offset, void* scratch, size_t scratch_bytes, int sms, cudaStream_t st);
size_t scan_scratch_bytes(int64_t n);
// Exclusive scan of int32 counts into uint64 offsets; also writes the total
// into offsets_total (device, may be null).
cudaError_t exclusive_scan_counts(const int32_t* counts, int64_t n, uint64_t* offsets, uint64_t* total, void* scratch,
                                  int sms, cudaStream_t st);
// Cell keys of positions with `dims` (2 or 3) coordinates; for 2 the third
// dimension has nx[2] == 1 and is not read.
cudaError_t cartesian_keys(const DField& pos, int dims, int64_t begin, int64_t end, const double* mn,
                           const double* rdx, const int32_t* nx, uint32_t* keys, int32_t* counts, int* error_flag,
                           cudaStream_t st, int sms);
cudaError_t key_histogram(const int32_t* keys, int64_t begin, int64_t end, uint32_t* keys_out, int32_t* counts,
                          int32_t nbin, int* error_flag, cudaStream_t st, int sms);
// minmax[0..1] = min and max of keys[begin, end) ((INT_MAX, INT_MIN) when
// the range is empty).
cudaError_t key_minmax(const int32_t* keys, int64_t begin, int64_t end, int* minmax, cudaStream_t st, int sms);
// Kokkos::BinOp1D bins of keys[begin, end) counted into counts[nbins]; the
// sort key is the bin, or key - kmin when by_key.
cudaError_t key_bin1d(const int32_t* keys, int64_t begin, int64_t end, int kmin, double mul, int32_t nbins, bool by_key,
                      uint32_t* keys_out, int32_t* counts, cudaStream_t st, int sms);
cudaError_t permute_field(const uint64_t* perm, int64_t begin, int64_t end, const DField& f, int ncomp, void* scratch,
                          cudaStream_t st, int sms);
cudaError_t tile_keys(const DMesh& mesh, const DField& pts, int64_t n, int order, const int32_t* tile,
                      const int32_t* num_tiles, uint32_t* keys, int32_t* tile_counts, cudaStream_t st, int sms);
// Work items of many instances in one list (instance-major): tile_offsets[i]
// (device array of device pointers) are instance i's tile offsets and
// tile_base (device, n_inst + 1 entries) the prefix sum of the instances'
// tile counts. Scratch: scan_scratch_bytes(total_tiles) + total_tiles * 4.
cudaError_t build_batch_work_items(const int64_t* const* tile_offsets, const int64_t* tile_base, int n_inst,
                                   int64_t total_tiles, int64_t chunk, int64_t* work_prefix, WorkItem* work,
                                   int64_t* work_count, void* scan_scratch, cudaStream_t st, int sms);
cudaError_t build_work_items(const int64_t* tile_offsets, int64_t num_tiles, int64_t chunk, int64_t* work_prefix,
                             WorkItem* work, int64_t* work_count, void* scan_scratch, cudaStream_t st, int sms);
cudaError_t counts_to_int64_offsets(const int32_t* counts, int64_t n, int64_t* offsets, void* scratch, cudaStream_t st,
                                    int sms);

}  // namespace cgx
