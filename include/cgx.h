/*
 * cgx -- C ABI of the GB300-native particle<->grid interpolation library.
 *
 * The entry points replace the device work of Cabana::Grid's interpolation
 * path. Each declaration names the reference interface it stands in for
 * (paths relative to the Cabana source tree).
 *
 * Conventions
 *   - All data pointers are device pointers unless stated otherwise. The
 *     caller owns every particle and grid buffer; the library never frees
 *     caller memory. Workspace (sort buffers, work lists) lives in a
 *     cgx_handle and is allocated on demand, grow-only.
 *   - Calls are asynchronous and stream-ordered on the `stream` argument
 *     (a cudaStream_t passed as void*; NULL = legacy default stream).
 *   - Every function returns a cgx_status; 0 is success. No C++ exception
 *     crosses this boundary. cgx_last_error() gives a message for the last
 *     failure on the calling thread.
 *   - A handle may be used by one host thread at a time.
 */
#ifndef CGX_H
#define CGX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int cgx_status;
#define CGX_OK 0
#define CGX_ERR_INVALID_ARG 1   /* bad pointer / size / kind (host check)      */
#define CGX_ERR_CUDA 2          /* a CUDA runtime call failed                   */
#define CGX_ERR_OUT_OF_BOUNDS 3 /* a stencil left the ghosted index space       */
#define CGX_ERR_TIMEOUT 4       /* a bounded device wait gave up                */
#define CGX_ERR_NOT_SUPPORTED 5 /* combination not built (e.g. spline order)   */
#define CGX_ERR_NO_MEMORY 6     /* workspace allocation failed                  */

/* Element types. */
#define CGX_F32 0
#define CGX_F64 1

/* Array entity types (Cabana::Grid::Node / Cell). */
#define CGX_NODE 0
#define CGX_CELL 1

/* Arithmetic forms of p2g / g2p.
 * CGX_PLAIN_FP64: one thread per point, double precision throughout, global
 *   atomics -- the arithmetic the reference's Kokkos CUDA path performs.
 * CGX_FP32_COMPENSATED: cell index and in-cell offset formed from the double
 *   coordinates to ~48-bit accuracy, spline weights and products in FP32,
 *   two-sum compensated per-tile accumulation, one atomic per node and dof
 *   at each tile flush. */
#define CGX_PLAIN_FP64 0
#define CGX_FP32_COMPENSATED 1

/* P2G operator kinds: the functors of
 * grid/src/Cabana_Grid_Interpolation.hpp:1324-1566. */
#define CGX_SCALAR_VALUE_P2G 0       /* ScalarValueP2G      :1324-1362 */
#define CGX_VECTOR_VALUE_P2G 1       /* VectorValueP2G      :1373-1413 */
#define CGX_SCALAR_GRADIENT_P2G 2    /* ScalarGradientP2G   :1424-1462 */
#define CGX_VECTOR_DIVERGENCE_P2G 3  /* VectorDivergenceP2G :1473-1513 */
#define CGX_TENSOR_DIVERGENCE_P2G 4  /* TensorDivergenceP2G :1524-1566 */
/* No reference counterpart: TensorDivergenceP2G of the transposed tensor,
 * grid_m += sum_n dW/dx_n * f[n][m]. It is the grid adjoint of
 * VectorGradientG2P (cgx_g2p_adjoint). */
#define CGX_TENSOR_DIVERGENCE_T_P2G 5

/* G2P operator kinds: the functors of
 * grid/src/Cabana_Grid_Interpolation.hpp:938-1182. */
#define CGX_SCALAR_VALUE_G2P 0       /* ScalarValueG2P      :938-977   */
#define CGX_VECTOR_VALUE_G2P 1       /* VectorValueG2P      :988-1028  */
#define CGX_SCALAR_GRADIENT_G2P 2    /* ScalarGradientG2P   :1039-1079 */
#define CGX_VECTOR_GRADIENT_G2P 3    /* VectorGradientG2P   :1090-1132 */
#define CGX_VECTOR_DIVERGENCE_G2P 4  /* VectorDivergenceG2P :1143-1182 */
/* No reference counterpart: VectorGradientG2P stored transposed,
 * x[m][n] += multiplier * sum dW/dx_n * f_m. It is the point-field adjoint of
 * TensorDivergenceP2G (cgx_p2g_adjoint). */
#define CGX_VECTOR_GRADIENT_T_G2P 5

/* Flags for cgx_p2g / cgx_g2p. */
#define CGX_FLAG_SKIP_HALO 1u     /* do not run the halo scatter / gather step   */
#define CGX_FLAG_CHECK_BOUNDS 2u  /* synchronise and report CGX_ERR_OUT_OF_BOUNDS */

/*
 * The uniform local mesh of one Array, reduced to scalars.
 * Stands in for LocalMesh<UniformMesh> (grid/src/Cabana_Grid_LocalMesh.hpp:
 * 61-120) plus the LocalGrid facts the halo needs
 * (grid/src/Cabana_Grid_LocalGrid_impl.hpp:49-60, :430-466).
 * Ghosted extents: owned_cells + 2*halo_width + (entity == CGX_NODE).
 *
 * num_space_dim 2 selects the 2D mesh (UniformMesh<double, 2>): entries [2]
 * of the per-dimension members are ignored, points hold 2 coordinates, an
 * Array is (i, j, dof), vector fields have 2 components and tensor fields
 * 2 x 2 (the 2D specialisations of grid/src/Cabana_Grid_Interpolation.hpp:
 * 81-98, :139-158, :212-237, :291-323, :373-396, :466-485, :527-547,
 * :597-621, :674-702, :756-788). 2D runs the point kernels only (no tiling,
 * adjoint or batched launches). 0 is read as 3.
 */
typedef struct cgx_mesh {
    double ghost_low[3];     /* LocalMesh::lowCorner(Ghost(), d)            */
    double cell_size[3];     /* GlobalMesh::cellSize(d)                     */
    int32_t owned_cells[3];  /* GlobalGrid::ownedNumCell(d)                 */
    int32_t halo_width;      /* LocalGrid::haloCellWidth()                  */
    int32_t periodic[3];     /* GlobalGrid::isPeriodic(d), one rank         */
    int32_t entity;          /* CGX_NODE / CGX_CELL of the arrays          */
    int32_t num_space_dim;   /* 3 (or 0) or 2                               */
    int32_t reserved;
} cgx_mesh;

/*
 * A per-point field: a Kokkos::View (p, ...) or a Cabana::Slice of an AoSoA.
 * Element (p, c) -- c the flattened component index, row-major over the
 * field's extra dimensions -- lives at element offset
 *     (p / vector_length) * soa_stride + (p % vector_length) + c * comp_stride
 * from `data`. A LayoutRight View (p, C) is {1, C, 1}; a LayoutLeft View is
 * {1, 1, n}; an AoSoA slice is {VL, sizeof(SoA)/sizeof(T), VL}
 * (core/src/Cabana_Slice.hpp:96-190, core/src/impl/Cabana_Index.hpp:61-80).
 */
typedef struct cgx_field {
    void* data;
    int32_t dtype;          /* CGX_F32 / CGX_F64                              */
    int32_t vector_length;  /* 1, or the AoSoA vector length (a power of two)  */
    int64_t soa_stride;
    int64_t comp_stride;
} cgx_field;

/* A grid Array: Kokkos::View<T****> (i, j, k, dof), LayoutRight, over the
 * ghosted entity index space (grid/src/Cabana_Grid_Array.hpp:44-300). */
typedef struct cgx_array {
    void* data;
    int32_t dtype;  /* CGX_F32 / CGX_F64 */
    int32_t dofs;   /* extent(3)         */
} cgx_array;

/* One operator functor: kind, multiplier, the point field it reads (P2G) or
 * accumulates into (G2P), and the grid array it scatters into (P2G) or
 * gathers from (G2P). */
typedef struct cgx_op {
    int32_t kind;
    int32_t reserved;
    double multiplier;
    cgx_field x;
    cgx_array array;
} cgx_op;

/*
 * Tile-major particle ordering, produced by cgx_sort_tiles and consumed by
 * the tiled kernels. Particles are grouped by the base node of their spline
 * stencil; tiles of tile[0] x tile[1] x tile[2] base nodes are numbered
 * i-major. Particles of tile t occupy [tile_offsets[t], tile_offsets[t+1])
 * of the sorted order. The ordering is a performance hint only: a point that
 * is not inside the tile it was filed under is still interpolated exactly.
 */
typedef struct cgx_tiling {
    int32_t tile[3];
    int32_t num_tiles[3];
    int32_t spline_order;
    int32_t reserved;
    int64_t* tile_offsets;  /* device, cgx_tiling_num_offsets() entries */
} cgx_tiling;

typedef struct cgx_context* cgx_handle;

/* ---- lifetime --------------------------------------------------------- */
cgx_status cgx_create(cgx_handle* out);
cgx_status cgx_destroy(cgx_handle h);
const char* cgx_last_error(void);
const char* cgx_version(void);

/* Kernel family used by the last cgx_p2g / cgx_g2p on this handle (no
 * reference counterpart; for tests and tuning). The tiled family needs
 * CGX_FP32_COMPENSATED, spline order 1-3 and a tiling with tile 8x8x8. */
#define CGX_DISPATCH_NONE 0
#define CGX_DISPATCH_POINTS 1
#define CGX_DISPATCH_TILED 2
int cgx_last_dispatch(cgx_handle h);

/* ---- interpolation ---------------------------------------------------- */

/*
 * Point-to-grid. Replaces Cabana::Grid::p2g(functor, points, num_point,
 * Spline<N>(), halo, array) (grid/src/Cabana_Grid_Interpolation.hpp:
 * 1217-1313), generalised to several functors sharing one spline evaluation
 * (the fused form of benchmark/grid/Cabana_Grid_InterpolationPerformance.cpp:
 * 48-69). Contributions are ADDED to the arrays; the caller zeroes them
 * (ArrayOp::assign). Afterwards the halo scatter(Sum) runs on each distinct
 * array unless CGX_FLAG_SKIP_HALO is set (a no-op on non-periodic meshes).
 * `points` must hold double coordinates. `tiling` may be NULL (one thread
 * per point, any order); with a tiling built for this mesh and order and
 * precision CGX_FP32_COMPENSATED the tiled kernel runs.
 */
cgx_status cgx_p2g(cgx_handle h, const cgx_mesh* mesh, const cgx_field* points,
                   int64_t num_point, int spline_order, const cgx_op* ops,
                   int n_ops, int precision, const cgx_tiling* tiling,
                   unsigned flags, void* stream);

/*
 * Grid-to-point. Replaces Cabana::Grid::g2p(array, halo, points, num_point,
 * Spline<N>(), functor) (grid/src/Cabana_Grid_Interpolation.hpp:831-927),
 * several functors per launch. The halo gather(Replace) runs first on each
 * distinct array unless CGX_FLAG_SKIP_HALO is set. Results are ADDED to the
 * point fields: x += multiplier * result.
 */
cgx_status cgx_g2p(cgx_handle h, const cgx_mesh* mesh, const cgx_field* points,
                   int64_t num_point, int spline_order, const cgx_op* ops,
                   int n_ops, int precision, const cgx_tiling* tiling,
                   unsigned flags, void* stream);

/*
 * Fused grid-to-point-to-grid: the g2p2g composition of
 * benchmark/grid/Cabana_Grid_InterpolationPerformance.cpp:129-174 (there a
 * benchmark-local function; no library counterpart), generalised to several
 * functors. Per point, one spline evaluation; the G2P functors add
 * multiplier * result into their point fields, then the P2G functors
 * scatter, reading point fields that may hold the values just gathered.
 * G2P reads every array as it was at the call: an array that is also a P2G
 * target is read from a snapshot taken first, so the result does not depend
 * on the order in which points run (the reference benchmark reads and
 * scatters into one array concurrently). Halo gather on the G2P arrays
 * before, scatter(Sum) on the P2G arrays after, unless CGX_FLAG_SKIP_HALO.
 * 3D meshes; >= 1 functor of each direction, 8 in all. Without a tiling
 * (or in the plain FP64 form) one fused point kernel runs; with a tiling
 * that the tiled kernels take (as for cgx_p2g) the tiled G2P launch then
 * the tiled P2G launch run, which gives the same results faster because
 * their shared-memory node boxes avoid per-point global atomics.
 */
cgx_status cgx_g2p2g(cgx_handle h, const cgx_mesh* mesh,
                     const cgx_field* points, int64_t num_point,
                     int spline_order, const cgx_op* g2p_ops, int n_g2p,
                     const cgx_op* p2g_ops, int n_p2g, int precision,
                     const cgx_tiling* tiling, unsigned flags, void* stream);

/* ---- batched launches (no reference counterpart) ----------------------- */

/*
 * One independent problem of a batch: its own mesh, its points in the tile
 * order of its own tiling (cgx_tiling_init + cgx_sort_tiles, tile 8x8x8,
 * the batch's spline order), and the point field and grid array of each
 * operator of the batch. Every instance uses the same operator kinds and
 * multipliers; operators that share an array in one instance must share it
 * in all, and an operator's array has the same dofs and dtype everywhere.
 */
#define CGX_BATCH_MAX_OPS 8
typedef struct cgx_instance {
    cgx_mesh mesh;
    cgx_field points;
    int64_t num_point;
    cgx_tiling tiling;
    cgx_field x[CGX_BATCH_MAX_OPS];
    cgx_array array[CGX_BATCH_MAX_OPS];
} cgx_instance;

typedef struct cgx_batch* cgx_batch_plan;

/*
 * Plan a batched p2g (p2g != 0) or g2p over n_inst instances with the
 * FP32-compensated tiled kernels (spline order 1-3, FP32 point fields for
 * g2p). `ops` give the kinds and multipliers; their x / array members are
 * ignored. The plan uploads the instance table, allocates its work lists
 * and prepares the kernels; it holds the pointers of `inst`, so the buffers
 * must outlive it (their contents may change, e.g. a re-sort with
 * cgx_sort_tiles into the same tile_offsets).
 */
cgx_status cgx_batch_plan_create(cgx_handle h, const cgx_instance* inst,
                                 int n_inst, int spline_order,
                                 const cgx_op* ops, int n_ops, int p2g,
                                 cgx_batch_plan* out);
cgx_status cgx_batch_plan_destroy(cgx_batch_plan plan);

/*
 * Run the plan on `stream`: one work-list build over all instances and one
 * persistent launch (g2p: one per distinct array), plus the single-rank
 * halo step of periodic instances unless CGX_FLAG_SKIP_HALO is set. P2G adds
 * into the arrays and G2P into the point fields, as cgx_p2g / cgx_g2p do.
 * Without CGX_FLAG_CHECK_BOUNDS the call neither allocates nor synchronises,
 * so it can be captured into a CUDA graph.
 */
cgx_status cgx_batch_execute(cgx_batch_plan plan, unsigned flags, void* stream);

/*
 * Autotune the plan on its own data: time each candidate (particles per
 * work item x resident CTAs per SM) with CUDA events and keep the fastest.
 * It runs the plan several times, so a p2g plan's arrays (or a g2p plan's
 * point fields) hold accumulated results afterwards: reset them before use.
 * best_ms (may be NULL) receives the best time of one execution.
 */
cgx_status cgx_batch_autotune(cgx_batch_plan plan, void* stream, double* best_ms);

/* The plan's current settings. */
cgx_status cgx_batch_get_config(cgx_batch_plan plan, int64_t* item_particles,
                                int* ctas_per_sm);
cgx_status cgx_batch_set_config(cgx_batch_plan plan, int64_t item_particles,
                                int ctas_per_sm);

/* ---- adjoints (no reference counterpart) ------------------------------ */

/*
 * One operator of an adjoint call: the forward operator (kind, multiplier)
 * and the forward and cotangent buffers it touches. For cgx_p2g_adjoint the
 * kind is a P2G kind; `x` is the forward input field (read for the position
 * adjoint), `x_bar` receives dL/dx (ADDED; data NULL skips it), `array_bar`
 * holds dL/d(forward array) (read) and `array` is unused. For cgx_g2p_adjoint
 * the kind is a G2P kind; `x_bar` holds dL/d(forward output field) (read),
 * `array` is the forward array (read for the position adjoint), `array_bar`
 * receives dL/d(array) (ADDED; data NULL skips it) and `x` is unused.
 */
typedef struct cgx_adjoint_op {
    int32_t kind;
    int32_t reserved;
    double multiplier;
    cgx_field x;
    cgx_field x_bar;
    cgx_array array;
    cgx_array array_bar;
} cgx_adjoint_op;

/*
 * Reverse-mode derivative of cgx_p2g for the same points, order and ops.
 * Point fields: dL/dx = multiplier * G2P of array_bar with the transposed
 * operator (ScalarValue -> ScalarValueG2P, VectorValue -> VectorValueG2P,
 * ScalarGradient -> VectorDivergenceG2P, VectorDivergence ->
 * ScalarGradientG2P, TensorDivergence -> CGX_VECTOR_GRADIENT_T_G2P); it runs
 * on the tiled kernels when `tiling` allows, as cgx_g2p does. Positions:
 * dL/d(points) is ADDED to `points_bar` (n x 3, any cgx_field layout; NULL
 * skips it), from the spline gradient (value operators) or Hessian
 * (gradient and divergence operators). On periodic meshes the adjoint of
 * the halo scatter(Sum) runs first, in place on each distinct array_bar
 * (ghost += its owned image), unless CGX_FLAG_SKIP_HALO is set.
 */
cgx_status cgx_p2g_adjoint(cgx_handle h, const cgx_mesh* mesh,
                           const cgx_field* points, int64_t num_point,
                           int spline_order, const cgx_adjoint_op* ops,
                           int n_ops, int precision, const cgx_tiling* tiling,
                           const cgx_field* points_bar, unsigned flags,
                           void* stream);

/*
 * Reverse-mode derivative of cgx_g2p. Grid: array_bar += P2G of x_bar with
 * the transposed operator (ScalarValue -> ScalarValueP2G, VectorValue ->
 * VectorValueP2G, ScalarGradient -> VectorDivergenceP2G, VectorGradient ->
 * CGX_TENSOR_DIVERGENCE_T_P2G, VectorDivergence -> ScalarGradientP2G), then,
 * on periodic meshes, the adjoint of the halo gather: every ghost of
 * array_bar that has an owned image is added to that image and cleared
 * (ghosts must hold no other cotangent on entry). Positions: as
 * cgx_p2g_adjoint, using `array` as the forward array after its gather.
 */
cgx_status cgx_g2p_adjoint(cgx_handle h, const cgx_mesh* mesh,
                           const cgx_field* points, int64_t num_point,
                           int spline_order, const cgx_adjoint_op* ops,
                           int n_ops, int precision, const cgx_tiling* tiling,
                           const cgx_field* points_bar, unsigned flags,
                           void* stream);

/* Halo::scatter(exec, ScatterReduce::Sum(), array) and Halo::gather(exec,
 * array) for NodeHaloPattern<3> on one rank (grid/src/Cabana_Grid_HaloBase.hpp:
 * 202-760, grid/src/impl/Cabana_Grid_Halo_Mpi.hpp:60-245): periodic
 * dimensions fold ghosts into (or fill ghosts from) their owned images;
 * non-periodic dimensions have no neighbour and are left alone. */
cgx_status cgx_halo_scatter_sum(const cgx_mesh* mesh, const cgx_array* array,
                                void* stream);
cgx_status cgx_halo_gather(const cgx_mesh* mesh, const cgx_array* array,
                           void* stream);

/* ArrayOp::assign(array, value, Ghost()) (grid/src/Cabana_Grid_Array.hpp:
 * 431-447) over the whole ghosted array. */
cgx_status cgx_array_assign(const cgx_mesh* mesh, const cgx_array* array,
                            double value, void* stream);

/* ---- binning ---------------------------------------------------------- */

/* CartesianGrid::init cell counts (core/src/impl/Cabana_CartesianGrid.hpp:
 * 61-73). Host only. */
cgx_status cgx_cartesian_num_bins(const double grid_min[3],
                                  const double grid_max[3],
                                  const double grid_delta[3],
                                  int32_t nbin_out[3]);

/*
 * LinkedCellList::build over [begin, end) (core/src/Cabana_LinkedCellList.hpp:
 * 652-745): counts[prod(nbin)], offsets[prod(nbin)] (exclusive scan of counts,
 * relative to `begin`), permutes[end-begin] (original indices in binned
 * order). Within a bin, particles keep ascending index order -- the order of
 * the reference's Serial backend -- so the output is deterministic. A
 * position outside [grid_min, grid_max] (the reference indexes out of bounds
 * there) is put in the nearest edge bin; the call stays asynchronous and
 * does not report it.
 */
cgx_status cgx_linked_cell_build(cgx_handle h, const cgx_field* positions,
                                 int64_t begin, int64_t end,
                                 const double grid_min[3],
                                 const double grid_max[3],
                                 const double grid_delta[3], int32_t* counts,
                                 uint64_t* offsets, uint64_t* permutes,
                                 void* stream);

/*
 * The same for LinkedCellList<MemorySpace, Scalar, 2> (2D positions (p, 0..1),
 * core/src/Cabana_LinkedCellList.hpp:652-745 with
 * core/src/impl/Cabana_CartesianGrid.hpp's 2D locatePoint :158-168 and
 * cardinalCellIndex :233-238, i * nbin[1] + j). counts / offsets hold
 * nbin[0] * nbin[1] bins; nbin[d] = floor((grid_max[d] - grid_min[d]) /
 * grid_delta[d]) as in cgx_cartesian_num_bins.
 */
cgx_status cgx_linked_cell_build_2d(cgx_handle h, const cgx_field* positions,
                                    int64_t begin, int64_t end,
                                    const double grid_min[2],
                                    const double grid_max[2],
                                    const double grid_delta[2],
                                    int32_t* counts, uint64_t* offsets,
                                    uint64_t* permutes, void* stream);

/* Binning by bin index: keys[begin..end) are bin numbers in [0, nbin),
 * counts[nbin], offsets[nbin], permutes[end-begin], stable in-bin order. The
 * BinSort of core/src/Cabana_Sort.hpp:164-182 with the identity as the bin
 * map (the tiled kernels' tile ordering uses the same sort); a key outside
 * [0, nbin) returns CGX_ERR_INVALID_ARG. */
cgx_status cgx_bin_by_key(cgx_handle h, const int32_t* keys, int64_t begin,
                          int64_t end, int32_t nbin, int32_t* counts,
                          uint64_t* offsets, uint64_t* permutes, void* stream);

/*
 * Cabana::binByKey(keys, nbin, begin, end) (sort_within_bins = 0) and
 * Cabana::sortByKey(keys, begin, end) (nbin = (end - begin) / 2,
 * sort_within_bins = 1) over int keys (core/src/Cabana_Sort.hpp:217-235,
 * :364-443): Kokkos::BinOp1D splits [min, max] of keys[begin..end) into
 * nbin + 1 bins, bin = int(mul * (key - min)) with mul = nbin / (max - min),
 * or 1 when max - min <= nbin. counts and offsets hold nbin + 1 entries;
 * permutes[end-begin] lists the entries by bin, then (sort_within_bins) by
 * key, then by index -- a deterministic instance of the reference's order,
 * whose in-bin order the parallel backends leave open. Reads the key range
 * back to the host, so the call synchronises `stream` (as the reference's
 * key reduction blocks) and cannot be captured in a CUDA graph.
 */
cgx_status cgx_bin_by_key_range(cgx_handle h, const int32_t* keys,
                                int64_t begin, int64_t end, int32_t nbin,
                                int sort_within_bins, int32_t* counts,
                                uint64_t* offsets, uint64_t* permutes,
                                void* stream);

/*
 * cgx_bin_by_key without any device allocation (no counterpart in the
 * reference). Same results as cgx_bin_by_key, for callers that may not let a
 * library allocate device memory: hosts whose device memory is owned and
 * budgeted by another allocator, or latency-bound loops where an allocation
 * (which can synchronise the device) is not allowed. Needs no handle.
 *
 * Its scratch is a fixed 6 MiB device array compiled into libcgx, held by
 * every GPU that loads the library until the process exits. Limits:
 * end - begin <= CGX_STATIC_MAX_KEYS and nbin <= CGX_STATIC_MAX_BINS; larger
 * problems return CGX_ERR_INVALID_ARG (use cgx_bin_by_key). The first call on
 * a device (with that device current) looks up the array's device address;
 * make that first call before any stream capture. All calls on a device
 * share the array: calls that overlap on the GPU race, so serialise them.
 * The call synchronises `stream` to report keys outside [0, nbin).
 */
#define CGX_STATIC_MAX_KEYS 262144
#define CGX_STATIC_MAX_BINS 1048576
cgx_status cgx_bin_by_key_static(const int32_t* keys, int64_t begin,
                                 int64_t end, int32_t nbin, int32_t* counts,
                                 uint64_t* offsets, uint64_t* permutes,
                                 void* stream);

/*
 * permute(BinningData, AoSoA/Slice/View) (core/src/Cabana_Sort.hpp:549-720):
 * for each field, element i in [begin, end) becomes old element
 * permutes[i - begin], all components (ncomps[f] of them) moved together.
 * Elements are moved bit for bit, so a field's dtype only gives the element
 * size: CGX_F32 for any 4-byte member (float, int32), CGX_F64 for any 8-byte
 * member (double, int64).
 */
cgx_status cgx_permute(cgx_handle h, const uint64_t* permutes, int64_t begin,
                       int64_t end, const cgx_field* fields,
                       const int32_t* ncomps, int n_fields, void* stream);

/* ---- tile ordering for the tiled kernels (no reference counterpart:
 *      the reference p2g/g2p are order-agnostic) ------------------------ */

/* Fill the host-side fields of a tiling for a mesh / order / tile shape. */
cgx_status cgx_tiling_init(const cgx_mesh* mesh, int spline_order,
                           const int32_t tile[3], cgx_tiling* out);
int64_t cgx_tiling_num_offsets(const cgx_tiling* tiling);

/* Compute tile-major keys of the points, stable-sort them, write the gather
 * permutation (sorted[i] = original[permutes[i]]) and tiling->tile_offsets.
 * Apply the permutation to every particle field with cgx_permute. */
cgx_status cgx_sort_tiles(cgx_handle h, const cgx_mesh* mesh,
                          const cgx_field* points, int64_t num_point,
                          cgx_tiling* tiling, uint64_t* permutes,
                          void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CGX_H */
