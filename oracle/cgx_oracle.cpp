// FP64 CPU oracle (test infrastructure only; see cgx_oracle.hpp).
#include "cgx_oracle.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int kMaxKnot = 7;

// ---------------------------------------------------------------------------
// Spline<N>. Orders 0-3 follow the closed forms of
// grid/src/Cabana_Grid_Splines.hpp:36-452 term by term. Orders 4-6
// (Splines.hpp:454-938) are evaluated from the same centred cardinal
// B-spline with the Cox-de Boor recurrence instead of the expanded
// polynomials; the two agree to rounding.
// ---------------------------------------------------------------------------
int num_knot(int order) { return order + 1; }

// Splines.hpp mapToLogicalGrid: dual grid (+0.5) for even orders.
double map_to_logical(int order, double xp, double rdx, double low_x) {
    if (order % 2 == 0) return (xp - low_x) * rdx + 0.5;
    return (xp - low_x) * rdx;
}

// Splines.hpp offsets()/stencil(): first index = int(x0) - order/2 for even,
// int(x0) - (order-1)/2 for odd orders.
int first_offset(int order) { return order % 2 == 0 ? -(order / 2) : -((order - 1) / 2); }

void stencil(int order, double x0, int* idx) {
    int base = static_cast<int>(x0) + first_offset(order);
    for (int a = 0; a < num_knot(order); ++a) idx[a] = base + a;
}

// Uniform B-spline basis on one unit interval: b[j] = B_d(u + d - j).
void de_boor(int degree, double u, double* b) {
    b[0] = 1.0;
    for (int d = 1; d <= degree; ++d) {
        double nb[kMaxKnot + 1];
        for (int j = 0; j <= d; ++j) {
            double left = (j >= 1) ? (u + d - j) * b[j - 1] : 0.0;
            double right = (j <= d - 1) ? (1.0 + j - u) * b[j] : 0.0;
            nb[j] = (left + right) / d;
        }
        for (int j = 0; j <= d; ++j) b[j] = nb[j];
    }
}

void value(int order, double x0, double* v) {
    double xi = x0 - static_cast<int>(x0);
    switch (order) {
        case 0:  // Splines.hpp:95-100
            v[0] = 1.0;
            return;
        case 1: {  // Splines.hpp:176-187
            double xn = x0 - static_cast<int>(x0);
            v[0] = 1.0 - xn;
            v[1] = xn;
            return;
        }
        case 2: {  // Splines.hpp:281-298
            double nine_eights = 9.0 / 8.0;
            double xn = x0 - static_cast<int>(x0) + 0.5;
            v[0] = 0.5 * xn * xn - 1.5 * xn + nine_eights;
            xn -= 1.0;
            v[1] = -xn * xn + 0.75;
            xn -= 1.0;
            v[2] = 0.5 * xn * xn + 1.5 * xn + nine_eights;
            return;
        }
        case 3: {  // Splines.hpp:393-420
            double one_sixth = 1.0 / 6.0;
            double two_thirds = one_sixth * 4.0;
            double four_thirds = two_thirds * 2.0;
            double xn = x0 - static_cast<int>(x0) + 1.0;
            double xn2 = xn * xn;
            v[0] = -xn * xn2 * one_sixth + xn2 - 2.0 * xn + four_thirds;
            xn -= 1.0;
            xn2 = xn * xn;
            v[1] = 0.5 * xn * xn2 - xn2 + two_thirds;
            xn -= 1.0;
            xn2 = xn * xn;
            v[2] = -0.5 * xn * xn2 - xn2 + two_thirds;
            xn -= 1.0;
            xn2 = xn * xn;
            v[3] = xn * xn2 * one_sixth + xn2 + 2.0 * xn + four_thirds;
            return;
        }
        default:
            de_boor(order, xi, v);
            return;
    }
}

void gradient(int order, double x0, double rdx, double* g) {
    double xi = x0 - static_cast<int>(x0);
    switch (order) {
        case 0:  // Splines.hpp:112-117
            g[0] = 0.0;
            return;
        case 1:  // Splines.hpp:199-206
            g[0] = -rdx;
            g[1] = rdx;
            return;
        case 2: {  // Splines.hpp:310-324
            double xn = x0 - static_cast<int>(x0) + 0.5;
            g[0] = (xn - 1.5) * rdx;
            xn -= 1.0;
            g[1] = (-2.0 * xn) * rdx;
            xn -= 1.0;
            g[2] = (xn + 1.5) * rdx;
            return;
        }
        case 3: {  // Splines.hpp:432-451
            double xn = x0 - static_cast<int>(x0) + 1.0;
            g[0] = (-0.5 * xn * xn + 2.0 * xn - 2.0) * rdx;
            xn -= 1.0;
            g[1] = (1.5 * xn * xn - 2.0 * xn) * rdx;
            xn -= 1.0;
            g[2] = (-1.5 * xn * xn - 2.0 * xn) * rdx;
            xn -= 1.0;
            g[3] = (0.5 * xn * xn + 2.0 * xn + 2.0) * rdx;
            return;
        }
        default: {
            // d/du B_n(u + n - a) = B_{n-1}(u + n - a) - B_{n-1}(u + n - 1 - a)
            double b[kMaxKnot + 1];
            de_boor(order - 1, xi, b);
            for (int a = 0; a <= order; ++a) {
                double left = (a >= 1) ? b[a - 1] : 0.0;
                double right = (a <= order - 1) ? b[a] : 0.0;
                g[a] = (left - right) * rdx;
            }
            return;
        }
    }
}

// ---------------------------------------------------------------------------
// LocalMesh<UniformMesh> (LocalMesh.hpp:180-200) and evaluateSpline
// (Splines.hpp:1283-1342).
// ---------------------------------------------------------------------------
struct Spline3 {
    int order;
    int nk;
    double dx[3];
    double x[3];
    int s[3][kMaxKnot];
    double w[3][kMaxKnot];
    double g[3][kMaxKnot];
    double d[3][kMaxKnot];
};

void entity_coordinates(const oracle_mesh& m, int index, int dim, double& out) {
    if (m.entity == 1)  // Cell: ghost_low + (i + 0.5) * cell_size
        out = m.ghost_low[dim] + (double(index) + double(0.5)) * m.cell_size[dim];
    else  // Node: ghost_low + i * cell_size
        out = m.ghost_low[dim] + double(index) * m.cell_size[dim];
}

void evaluate(const oracle_mesh& m, int order, const double* p, Spline3& sd) {
    sd.order = order;
    sd.nk = num_knot(order);
    double low_x[3], low_x_p1[3], rdx[3];
    for (int d = 0; d < 3; ++d) {
        entity_coordinates(m, 0, d, low_x[d]);
        entity_coordinates(m, 1, d, low_x_p1[d]);
    }
    for (int d = 0; d < 3; ++d) sd.dx[d] = low_x_p1[d] - low_x[d];
    for (int d = 0; d < 3; ++d) rdx[d] = 1.0 / sd.dx[d];
    for (int d = 0; d < 3; ++d) sd.x[d] = map_to_logical(order, p[d], rdx[d], low_x[d]);
    for (int d = 0; d < 3; ++d) stencil(order, sd.x[d], sd.s[d]);
    for (int d = 0; d < 3; ++d) value(order, sd.x[d], sd.w[d]);
    for (int d = 0; d < 3; ++d) gradient(order, sd.x[d], rdx[d], sd.g[d]);
    // SplinePhysicalDistance (Splines.hpp:1233-1251)
    for (int d = 0; d < 3; ++d) {
        double offset = low_x[d] - p[d];
        for (int n = 0; n < sd.nk; ++n) sd.d[d][n] = offset + sd.s[d][n] * sd.dx[d];
    }
}

void extents(const oracle_mesh& m, int64_t* ext) {
    for (int d = 0; d < 3; ++d)
        ext[d] = int64_t(m.owned_cells[d]) + 2 * m.halo_width + (m.entity == 1 ? 0 : 1);
}

struct GridView {
    double* data;
    int64_t n0, n1, n2;
    int dofs;
    bool bad = false;
    double& at(int i, int j, int k, int dof) {
        return data[((int64_t(i) * n1 + j) * n2 + k) * dofs + dof];
    }
};

bool stencil_in_range(const Spline3& sd, const int64_t* ext) {
    for (int d = 0; d < 3; ++d) {
        if (sd.s[d][0] < 0 || sd.s[d][sd.nk - 1] >= ext[d]) return false;
    }
    return true;
}

// P2G:: thread-level operators, Interpolation.hpp:437-747 (3D).
void p2g_point(int kind, double mult, const double* xp, const Spline3& sd, GridView& v) {
    const int nk = sd.nk;
    switch (kind) {
        case 0: {  // ScalarValueP2G (Interpolation.hpp:1344-1351) -> P2G::value :437-458
            double pd = xp[0] * mult;
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int k = 0; k < nk; ++k)
                        v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], 0) +=
                            pd * sd.w[0][i] * sd.w[1][j] * sd.w[2][k];
            return;
        }
        case 1: {  // VectorValueP2G (:1393-1402) -> P2G::value :489-518
            double pd[3];
            for (int d = 0; d < 3; ++d) pd[d] = mult * xp[d];
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int k = 0; k < nk; ++k)
                        for (int d = 0; d < 3; ++d)
                            v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], d) +=
                                pd[d] * sd.w[0][i] * sd.w[1][j] * sd.w[2][k];
            return;
        }
        case 2: {  // ScalarGradientP2G (:1444-1451) -> P2G::gradient :557-588
            double pd = xp[0] * mult;
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int k = 0; k < nk; ++k) {
                        v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], 0) +=
                            pd * sd.g[0][i] * sd.w[1][j] * sd.w[2][k];
                        v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], 1) +=
                            pd * sd.w[0][i] * sd.g[1][j] * sd.w[2][k];
                        v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], 2) +=
                            pd * sd.w[0][i] * sd.w[1][j] * sd.g[2][k];
                    }
            return;
        }
        case 3: {  // VectorDivergenceP2G (:1493-1502) -> P2G::divergence :631-665
            double pd[3];
            for (int d = 0; d < 3; ++d) pd[d] = mult * xp[d];
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int k = 0; k < nk; ++k) {
                        double result = pd[0] * sd.g[0][i] * sd.w[1][j] * sd.w[2][k] +
                                        pd[1] * sd.w[0][i] * sd.g[1][j] * sd.w[2][k] +
                                        pd[2] * sd.w[0][i] * sd.w[1][j] * sd.g[2][k];
                        v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], 0) += result;
                    }
            return;
        }
        case 4: {  // TensorDivergenceP2G (:1544-1555) -> P2G::divergence :712-747
            double pd[3][3];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) pd[a][b] = mult * xp[a * 3 + b];
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int k = 0; k < nk; ++k) {
                        double rg[3] = {sd.g[0][i] * sd.w[1][j] * sd.w[2][k],
                                        sd.w[0][i] * sd.g[1][j] * sd.w[2][k],
                                        sd.w[0][i] * sd.w[1][j] * sd.g[2][k]};
                        for (int d1 = 0; d1 < 3; ++d1)
                            for (int d0 = 0; d0 < 3; ++d0)
                                v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], d0) +=
                                    rg[d1] * pd[d0][d1];
                    }
            return;
        }
    }
}

int p2g_comps(int kind) {
    switch (kind) {
        case 0: case 2: return 1;
        case 1: case 3: return 3;
        case 4: return 9;
    }
    return -1;
}
int g2p_comps(int kind) {
    switch (kind) {
        case 0: case 4: return 1;
        case 1: case 2: return 3;
        case 3: return 9;
    }
    return -1;
}

// G2P:: thread-level operators, Interpolation.hpp:53-364 (3D), applied by the
// functors at :938-1182 (x += multiplier * result).
void g2p_point(int kind, double mult, double* xp, const Spline3& sd, GridView& v) {
    const int nk = sd.nk;
    switch (kind) {
        case 0: {  // ScalarValueG2P -> G2P::value :53-72
            double result = 0.0;
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int k = 0; k < nk; ++k)
                        result += v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], 0) *
                                  sd.w[0][i] * sd.w[1][j] * sd.w[2][k];
            xp[0] += mult * result;
            return;
        }
        case 1: {  // VectorValueG2P -> G2P::value :108-130
            double result[3] = {0.0, 0.0, 0.0};
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int k = 0; k < nk; ++k)
                        for (int d = 0; d < 3; ++d)
                            result[d] += v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], d) *
                                         sd.w[0][i] * sd.w[1][j] * sd.w[2][k];
            for (int d = 0; d < 3; ++d) xp[d] += mult * result[d];
            return;
        }
        case 2: {  // ScalarGradientG2P -> G2P::gradient :168-203
            double result[3] = {0.0, 0.0, 0.0};
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int k = 0; k < nk; ++k) {
                        double f = v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], 0);
                        result[0] += f * sd.g[0][i] * sd.w[1][j] * sd.w[2][k];
                        result[1] += f * sd.w[0][i] * sd.g[1][j] * sd.w[2][k];
                        result[2] += f * sd.w[0][i] * sd.w[1][j] * sd.g[2][k];
                    }
            for (int d = 0; d < 3; ++d) xp[d] += mult * result[d];
            return;
        }
        case 3: {  // VectorGradientG2P -> G2P::gradient :247-282 (result[m][n] = d_m W * f_n)
            double result[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int k = 0; k < nk; ++k) {
                        double rg[3] = {sd.g[0][i] * sd.w[1][j] * sd.w[2][k],
                                        sd.w[0][i] * sd.g[1][j] * sd.w[2][k],
                                        sd.w[0][i] * sd.w[1][j] * sd.g[2][k]};
                        for (int d0 = 0; d0 < 3; ++d0) {
                            double mg = rg[d0];
                            for (int d1 = 0; d1 < 3; ++d1)
                                result[d0][d1] +=
                                    mg * v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], d1);
                        }
                    }
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) xp[a * 3 + b] += mult * result[a][b];
            return;
        }
        case 4: {  // VectorDivergenceG2P -> G2P::divergence :333-364
            double result = 0.0;
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int k = 0; k < nk; ++k)
                        result += v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], 0) *
                                      sd.g[0][i] * sd.w[1][j] * sd.w[2][k] +
                                  v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], 1) *
                                      sd.w[0][i] * sd.g[1][j] * sd.w[2][k] +
                                  v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], 2) *
                                      sd.w[0][i] * sd.w[1][j] * sd.g[2][k];
            xp[0] += result * mult;
            return;
        }
    }
}

// Node/cell halo on a single rank (HaloBase.hpp:202-760 with the shared index
// spaces of LocalGrid_impl.hpp:430-510). A ghost entity exchanges with an
// owned one only when every dimension in which it lies outside the owned
// range is periodic; the owned partner wraps by the owned cell count.
bool halo_partner(const oracle_mesh& m, const int64_t* ext, const int64_t* idx, int64_t* own) {
    bool ghost = false;
    for (int d = 0; d < 3; ++d) {
        const int64_t hw = m.halo_width, nc = m.owned_cells[d];
        const int64_t own_hi = m.periodic[d] ? hw + nc : hw + nc + (m.entity == 1 ? 0 : 1);
        if (idx[d] >= hw && idx[d] < own_hi) {
            own[d] = idx[d];
            continue;
        }
        if (!m.periodic[d]) return false;
        ghost = true;
        int64_t r = ((idx[d] - hw) % nc + nc) % nc;
        own[d] = hw + r;
    }
    (void)ext;
    return ghost;
}

}  // namespace

extern "C" {

int oracle_spline_num_knot(int order) { return num_knot(order); }

void oracle_spline_offsets(int order, int* offsets) {
    for (int a = 0; a < num_knot(order); ++a) offsets[a] = first_offset(order) + a;
}

double oracle_spline_map(int order, double xp, double rdx, double low_x) {
    return map_to_logical(order, xp, rdx, low_x);
}

void oracle_spline_stencil(int order, double x0, int* indices) { stencil(order, x0, indices); }
void oracle_spline_value(int order, double x0, double* values) { value(order, x0, values); }
void oracle_spline_gradient(int order, double x0, double rdx, double* grads) {
    gradient(order, x0, rdx, grads);
}

void oracle_evaluate_spline(const oracle_mesh* mesh, int order, const double* p, double* dx,
                            double* x, int* s, double* w, double* g, double* d) {
    Spline3 sd;
    evaluate(*mesh, order, p, sd);
    const int nk = sd.nk;
    for (int a = 0; a < 3; ++a) {
        dx[a] = sd.dx[a];
        x[a] = sd.x[a];
        for (int n = 0; n < nk; ++n) {
            s[a * nk + n] = sd.s[a][n];
            w[a * nk + n] = sd.w[a][n];
            g[a * nk + n] = sd.g[a][n];
            d[a * nk + n] = sd.d[a][n];
        }
    }
}

void oracle_extents(const oracle_mesh* mesh, int64_t* ext) { extents(*mesh, ext); }

void oracle_halo_scatter_sum(const oracle_mesh* mesh, double* array, int dofs) {
    int64_t ext[3];
    extents(*mesh, ext);
    GridView v{array, ext[0], ext[1], ext[2], dofs};
    // Packs are taken from the ghosts before any owned entity is updated
    // (Halo_Mpi.hpp:166-245); ghosts and owned entities are disjoint, so a
    // direct pass is equivalent.
    for (int64_t i = 0; i < ext[0]; ++i)
        for (int64_t j = 0; j < ext[1]; ++j)
            for (int64_t k = 0; k < ext[2]; ++k) {
                int64_t idx[3] = {i, j, k}, own[3];
                if (!halo_partner(*mesh, ext, idx, own)) continue;
                for (int c = 0; c < dofs; ++c)
                    v.at(own[0], own[1], own[2], c) += v.at(i, j, k, c);
            }
}

void oracle_halo_gather(const oracle_mesh* mesh, double* array, int dofs) {
    int64_t ext[3];
    extents(*mesh, ext);
    GridView v{array, ext[0], ext[1], ext[2], dofs};
    for (int64_t i = 0; i < ext[0]; ++i)
        for (int64_t j = 0; j < ext[1]; ++j)
            for (int64_t k = 0; k < ext[2]; ++k) {
                int64_t idx[3] = {i, j, k}, own[3];
                if (!halo_partner(*mesh, ext, idx, own)) continue;
                for (int c = 0; c < dofs; ++c) v.at(i, j, k, c) = v.at(own[0], own[1], own[2], c);
            }
}

// Global p2g, Interpolation.hpp:1221-1268. Points outside the ghosted index
// space are skipped (the reference leaves that undefined) and counted in the
// return value.
int oracle_p2g(const oracle_mesh* mesh, const double* points, int64_t num_point, int order,
               const oracle_op* ops, int n_ops, int nthreads) {
    int64_t ext[3];
    extents(*mesh, ext);
    int skipped = 0;
    if (nthreads <= 1) {
        std::vector<GridView> views;
        for (int o = 0; o < n_ops; ++o) views.push_back({ops[o].array, ext[0], ext[1], ext[2], ops[o].dofs});
        for (int64_t p = 0; p < num_point; ++p) {
            Spline3 sd;
            evaluate(*mesh, order, points + 3 * p, sd);
            if (!stencil_in_range(sd, ext)) { ++skipped; continue; }
            for (int o = 0; o < n_ops; ++o)
                p2g_point(ops[o].kind, ops[o].multiplier, ops[o].x + p * p2g_comps(ops[o].kind), sd, views[o]);
        }
    } else {
#ifdef _OPENMP
        // Duplicated ScatterView: every thread accumulates into a private
        // zeroed copy of each target array; contribute() then sums the
        // copies into the caller's arrays.
        const int64_t nnode = ext[0] * ext[1] * ext[2];
        std::vector<std::vector<double>> dup(size_t(nthreads) * n_ops);
        #pragma omp parallel num_threads(nthreads) reduction(+ : skipped)
        {
            const int t = omp_get_thread_num();
            std::vector<GridView> views;
            for (int o = 0; o < n_ops; ++o) {
                auto& buf = dup[size_t(t) * n_ops + o];
                buf.assign(size_t(nnode) * ops[o].dofs, 0.0);
                views.push_back({buf.data(), ext[0], ext[1], ext[2], ops[o].dofs});
            }
            #pragma omp for schedule(static)
            for (int64_t p = 0; p < num_point; ++p) {
                Spline3 sd;
                evaluate(*mesh, order, points + 3 * p, sd);
                if (!stencil_in_range(sd, ext)) { ++skipped; continue; }
                for (int o = 0; o < n_ops; ++o)
                    p2g_point(ops[o].kind, ops[o].multiplier, ops[o].x + p * p2g_comps(ops[o].kind), sd, views[o]);
            }
            #pragma omp barrier
            for (int o = 0; o < n_ops; ++o) {
                const int64_t len = nnode * ops[o].dofs;
                #pragma omp for schedule(static)
                for (int64_t e = 0; e < len; ++e) {
                    double s = 0.0;
                    for (int u = 0; u < nthreads; ++u) s += dup[size_t(u) * n_ops + o][e];
                    ops[o].array[e] += s;
                }
            }
        }
#endif
    }
    // halo.scatter(Sum) once per distinct target array.
    for (int o = 0; o < n_ops; ++o) {
        bool seen = false;
        for (int q = 0; q < o; ++q) seen |= (ops[q].array == ops[o].array);
        if (!seen) oracle_halo_scatter_sum(mesh, ops[o].array, ops[o].dofs);
    }
    return skipped;
}

// Global g2p, Interpolation.hpp:835-880: halo.gather then the point loop.
int oracle_g2p(const oracle_mesh* mesh, const double* points, int64_t num_point, int order,
               const oracle_op* ops, int n_ops, int nthreads) {
    int64_t ext[3];
    extents(*mesh, ext);
    for (int o = 0; o < n_ops; ++o) {
        bool seen = false;
        for (int q = 0; q < o; ++q) seen |= (ops[q].array == ops[o].array);
        if (!seen) oracle_halo_gather(mesh, ops[o].array, ops[o].dofs);
    }
    std::vector<GridView> views;
    for (int o = 0; o < n_ops; ++o) views.push_back({ops[o].array, ext[0], ext[1], ext[2], ops[o].dofs});
    int skipped = 0;
#ifdef _OPENMP
    #pragma omp parallel for schedule(static) num_threads(nthreads > 1 ? nthreads : 1) reduction(+ : skipped)
#endif
    for (int64_t p = 0; p < num_point; ++p) {
        Spline3 sd;
        evaluate(*mesh, order, points + 3 * p, sd);
        if (!stencil_in_range(sd, ext)) { ++skipped; continue; }
        for (int o = 0; o < n_ops; ++o) {
            GridView v = views[o];
            g2p_point(ops[o].kind, ops[o].multiplier, ops[o].x + p * g2p_comps(ops[o].kind), sd, v);
        }
    }
    return skipped;
}

// CartesianGrid::init, Cabana_CartesianGrid.hpp:61-73 and cellsBetween :279-283.
void oracle_cartesian_num_bins(const double* grid_min, const double* grid_max,
                               const double* grid_delta, int32_t* nbin) {
    for (int d = 0; d < 3; ++d)
        nbin[d] = static_cast<int32_t>(std::floor((grid_max[d] - grid_min[d]) * (1.0 / grid_delta[d])));
}

// LinkedCellList::build, Cabana_LinkedCellList.hpp:652-745, run serially so
// that particles inside a bin keep ascending index order.
void oracle_linked_cell_build(const double* positions, int64_t begin, int64_t end,
                              const double* grid_min, const double* grid_max,
                              const double* grid_delta, int32_t* counts, uint64_t* offsets,
                              uint64_t* permutes) {
    int32_t nx[3];
    double dx[3], rdx[3];
    oracle_cartesian_num_bins(grid_min, grid_max, grid_delta, nx);
    for (int d = 0; d < 3; ++d) {
        dx[d] = (grid_max[d] - grid_min[d]) / nx[d];
        rdx[d] = 1.0 / dx[d];
    }
    const int64_t ncell = int64_t(nx[0]) * nx[1] * nx[2];
    auto cell_of = [&](int64_t p) {
        int c[3];
        for (int d = 0; d < 3; ++d) {
            // locatePoint, CartesianGrid.hpp:171-182
            c[d] = static_cast<int>(std::floor((positions[3 * p + d] - grid_min[d]) * rdx[d]));
            c[d] = (c[d] == nx[d]) ? c[d] - 1 : c[d];
        }
        // cardinalCellIndex, CartesianGrid.hpp:226-231
        return (int64_t(c[0]) * nx[1] + c[1]) * nx[2] + c[2];
    };
    std::fill(counts, counts + ncell, 0);
    for (int64_t p = begin; p < end; ++p) counts[cell_of(p)] += 1;
    uint64_t run = 0;
    for (int64_t c = 0; c < ncell; ++c) {
        offsets[c] = run;
        run += counts[c];
    }
    std::vector<int32_t> fill(ncell, 0);
    for (int64_t p = begin; p < end; ++p) {
        int64_t c = cell_of(p);
        permutes[offsets[c] + fill[c]++] = uint64_t(p);
    }
}

void oracle_bin_by_key(const int32_t* keys, int64_t begin, int64_t end, int32_t nbin,
                       int32_t* counts, uint64_t* offsets, uint64_t* permutes) {
    std::fill(counts, counts + nbin, 0);
    for (int64_t p = begin; p < end; ++p) counts[keys[p]] += 1;
    uint64_t run = 0;
    for (int32_t c = 0; c < nbin; ++c) {
        offsets[c] = run;
        run += counts[c];
    }
    std::vector<int32_t> fill(nbin, 0);
    for (int64_t p = begin; p < end; ++p) {
        int32_t c = keys[p];
        permutes[offsets[c] + fill[c]++] = uint64_t(p);
    }
}

// permute(BinningData, ...) Sort.hpp:549-588: gather into scratch, copy back.
void oracle_permute(const uint64_t* permutes, int64_t begin, int64_t end, double* data, int comps) {
    std::vector<double> scratch(size_t(end - begin) * comps);
    for (int64_t i = begin; i < end; ++i)
        for (int c = 0; c < comps; ++c)
            scratch[size_t(i - begin) * comps + c] = data[int64_t(permutes[i - begin]) * comps + c];
    for (int64_t i = begin; i < end; ++i)
        for (int c = 0; c < comps; ++c) data[i * comps + c] = scratch[size_t(i - begin) * comps + c];
}

void oracle_stable_sort_keys(const uint64_t* keys, int64_t n, uint64_t* permutes) {
    std::vector<uint64_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return keys[a] < keys[b]; });
    std::copy(idx.begin(), idx.end(), permutes);
}

}  // extern "C"
