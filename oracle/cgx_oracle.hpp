// FP64 CPU oracle for the particle<->grid interpolation path.
//
// TEST INFRASTRUCTURE ONLY. This library is the checker: the parity tests,
// the smoke check and the CPU-baseline leg of the benchmark link it. The
// product path (libcgx.so) never calls into it.
//
// It is a restatement, in plain C++17, of the reference algorithms:
//   * Spline<N> mapping / stencil / value / gradient
//       grid/src/Cabana_Grid_Splines.hpp:30-938
//   * SplineData + evaluateSpline
//       grid/src/Cabana_Grid_Splines.hpp:1051-1342
//   * uniform LocalMesh coordinates
//       grid/src/Cabana_Grid_LocalMesh.hpp:61-200
//   * G2P:: / P2G:: thread-level operators (3D)
//       grid/src/Cabana_Grid_Interpolation.hpp:53-747
//   * the ten operator functors and the global p2g / g2p drivers
//       grid/src/Cabana_Grid_Interpolation.hpp:831-1566
//   * single-rank node halo scatter(Sum) / gather(Replace)
//       grid/src/Cabana_Grid_HaloBase.hpp:202-760,
//       grid/src/Cabana_Grid_LocalGrid_impl.hpp:430-510
//   * CartesianGrid + LinkedCellList::build (serial order)
//       core/src/impl/Cabana_CartesianGrid.hpp:61-283,
//       core/src/Cabana_LinkedCellList.hpp:652-745
//   * BinningData + permute
//       core/src/Cabana_Sort.hpp:37-136, :549-720
//
// Everything runs in double precision. Floating-point contraction is
// disabled at compile time so results do not depend on the host ISA.
#pragma once
#include <cstdint>

extern "C" {

// Mesh description shared with the product ABI (same field meaning as
// cgx_mesh in include/cgx.h).
typedef struct oracle_mesh {
    double ghost_low[3];
    double cell_size[3];
    int32_t owned_cells[3];
    int32_t halo_width;
    int32_t periodic[3];
    int32_t entity;  // 0 = Node, 1 = Cell
    int32_t num_space_dim;  // 3 (or 0) or 2: entries [2] are then ignored
    int32_t reserved;
} oracle_mesh;

// One operator. `x` is a dense row-major (num_point, comps) double array,
// `array` the dense (i, j, k, dof) double grid array over the ghosted
// index space.
typedef struct oracle_op {
    int32_t kind;
    int32_t dofs;
    double multiplier;
    double* x;
    double* array;
} oracle_op;

int oracle_spline_num_knot(int order);
void oracle_spline_offsets(int order, int* offsets);
double oracle_spline_map(int order, double xp, double rdx, double low_x);
void oracle_spline_stencil(int order, double x0, int* indices);
void oracle_spline_value(int order, double x0, double* values);
void oracle_spline_gradient(int order, double x0, double rdx, double* grads);

// evaluateSpline for one point. Outputs are [3][num_knot] row-major.
void oracle_evaluate_spline(const oracle_mesh* mesh, int order,
                            const double* p, double* dx, double* x, int* s,
                            double* w, double* g, double* d);

// Ghosted entity extents of the mesh (Node: cells + 2 hw + 1).
void oracle_extents(const oracle_mesh* mesh, int64_t* ext);

// Global p2g / g2p, including the halo step. nthreads > 1 runs the
// OpenMP restatement that mirrors a duplicated Kokkos ScatterView.
int oracle_p2g(const oracle_mesh* mesh, const double* points,
               int64_t num_point, int order, const oracle_op* ops, int n_ops,
               int nthreads);
int oracle_g2p(const oracle_mesh* mesh, const double* points,
               int64_t num_point, int order, const oracle_op* ops, int n_ops,
               int nthreads);

// Fused g2p2g: per point the G2P functors (reading each array as it was at
// the call) then the P2G functors; halo gather before, scatter after.
int oracle_g2p2g(const oracle_mesh* mesh, const double* points,
                 int64_t num_point, int order, const oracle_op* g2p_ops,
                 int n_g2p, const oracle_op* p2g_ops, int n_p2g);

void oracle_halo_scatter_sum(const oracle_mesh* mesh, double* array,
                             int dofs);
void oracle_halo_gather(const oracle_mesh* mesh, double* array, int dofs);

// CartesianGrid::init arithmetic: number of bins per dimension.
void oracle_cartesian_num_bins(const double* grid_min, const double* grid_max,
                               const double* grid_delta, int32_t* nbin);
// LinkedCellList::build over [begin, end) of a dense (n, 3) position array,
// serial order. counts/offsets have prod(nbin) entries, permutes end-begin.
void oracle_linked_cell_build(const double* positions, int64_t begin,
                              int64_t end, const double* grid_min,
                              const double* grid_max,
                              const double* grid_delta, int32_t* counts,
                              uint64_t* offsets, uint64_t* permutes);
// binByKey equivalent with a stable in-bin order.
void oracle_bin_by_key(const int32_t* keys, int64_t begin, int64_t end,
                       int32_t nbin, int32_t* counts, uint64_t* offsets,
                       uint64_t* permutes);
// permute(BinningData, data) for a dense (n, comps) double array.
void oracle_permute(const uint64_t* permutes, int64_t begin, int64_t end,
                    double* data, int comps);

// Second derivatives of the knot weights in the physical coordinate.
void oracle_spline_hessian(int order, double x0, double rdx, double* h);

// One operator of an adjoint call: dense (n, comps) point arrays and dense
// (i, j, k, dof) grid arrays. P2G adjoint: x = forward input (read; NULL
// skips the position term), x_bar = dL/dx (added; may be NULL), array_bar =
// dL/d(array) (read; halo-adjusted in place). G2P adjoint: x_bar =
// dL/d(output) (read), array = forward array (read; NULL skips the position
// term), array_bar = dL/d(array) (added; may be NULL).
typedef struct oracle_adjoint_op {
    int32_t kind;
    int32_t dofs;
    double multiplier;
    double* x;
    double* x_bar;
    double* array;
    double* array_bar;
} oracle_adjoint_op;

// Reverse-mode derivatives of oracle_p2g / oracle_g2p; points_bar (n, 3)
// receives dL/d(position), added (may be NULL). Return the skipped count.
int oracle_p2g_adjoint(const oracle_mesh* mesh, const double* points,
                       int64_t num_point, int order,
                       const oracle_adjoint_op* ops, int n_ops,
                       double* points_bar);
int oracle_g2p_adjoint(const oracle_mesh* mesh, const double* points,
                       int64_t num_point, int order,
                       const oracle_adjoint_op* ops, int n_ops,
                       double* points_bar);

// Stable key sort used to order particles tile by tile; returns the gather
// permutation.
void oracle_stable_sort_keys(const uint64_t* keys, int64_t n,
                             uint64_t* permutes);
}
