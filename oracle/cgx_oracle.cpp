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

// Second derivatives of the knot weights in the physical coordinate (no
// reference counterpart; the reference has value and gradient only): the
// derivative of gradient() above. Orders 2 and 3 differentiate the closed
// forms; higher orders use d2/du2 B_n = B_{n-2}[a-2] - 2 B_{n-2}[a-1] + B_{n-2}[a].
void hessian(int order, double x0, double rdx, double* h) {
    const double xi = x0 - static_cast<int>(x0);
    const double r2 = rdx * rdx;
    switch (order) {
        case 0:
            h[0] = 0.0;
            return;
        case 1:
            h[0] = h[1] = 0.0;
            return;
        case 2:  // d/dxn of (xn - 1.5), (-2 xn), (xn + 1.5)
            h[0] = r2;
            h[1] = -2.0 * r2;
            h[2] = r2;
            return;
        case 3: {  // d/dxn of the four gradient polynomials
            double xn = xi + 1.0;
            h[0] = (-xn + 2.0) * r2;
            xn -= 1.0;
            h[1] = (3.0 * xn - 2.0) * r2;
            xn -= 1.0;
            h[2] = (-3.0 * xn - 2.0) * r2;
            xn -= 1.0;
            h[3] = (xn + 2.0) * r2;
            return;
        }
        default: {
            double b[kMaxKnot + 1];
            de_boor(order - 2, xi, b);
            for (int a = 0; a <= order; ++a) {
                const double l2 = (a >= 2) ? b[a - 2] : 0.0;
                const double l1 = (a >= 1 && a - 1 <= order - 2) ? b[a - 1] : 0.0;
                const double l0 = (a <= order - 2) ? b[a] : 0.0;
                h[a] = (l2 - 2.0 * l1 + l0) * r2;
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

// Number of space dimensions of a mesh (num_space_dim 0 reads as 3).
int dims(const oracle_mesh& m) { return m.num_space_dim == 2 ? 2 : 3; }

void entity_coordinates(const oracle_mesh& m, int index, int dim, double& out) {
    if (m.entity == 1)  // Cell: ghost_low + (i + 0.5) * cell_size
        out = m.ghost_low[dim] + (double(index) + double(0.5)) * m.cell_size[dim];
    else  // Node: ghost_low + i * cell_size
        out = m.ghost_low[dim] + double(index) * m.cell_size[dim];
}

// The point p holds dims(m) coordinates; in 2D the third dimension's
// members are left zero.
void evaluate(const oracle_mesh& m, int order, const double* p, Spline3& sd) {
    const int nd = dims(m);
    sd = Spline3{};
    sd.order = order;
    sd.nk = num_knot(order);
    double low_x[3], low_x_p1[3], rdx[3];
    for (int d = 0; d < nd; ++d) {
        entity_coordinates(m, 0, d, low_x[d]);
        entity_coordinates(m, 1, d, low_x_p1[d]);
    }
    for (int d = 0; d < nd; ++d) sd.dx[d] = low_x_p1[d] - low_x[d];
    for (int d = 0; d < nd; ++d) rdx[d] = 1.0 / sd.dx[d];
    for (int d = 0; d < nd; ++d) sd.x[d] = map_to_logical(order, p[d], rdx[d], low_x[d]);
    for (int d = 0; d < nd; ++d) stencil(order, sd.x[d], sd.s[d]);
    for (int d = 0; d < nd; ++d) value(order, sd.x[d], sd.w[d]);
    for (int d = 0; d < nd; ++d) gradient(order, sd.x[d], rdx[d], sd.g[d]);
    // SplinePhysicalDistance (Splines.hpp:1233-1251)
    for (int d = 0; d < nd; ++d) {
        double offset = low_x[d] - p[d];
        for (int n = 0; n < sd.nk; ++n) sd.d[d][n] = offset + sd.s[d][n] * sd.dx[d];
    }
}

// Ghosted entity extents; a 2D mesh has one layer in the third dimension so
// its (i, j, dof) arrays index as (i, j, 0, dof).
void extents(const oracle_mesh& m, int64_t* ext) {
    for (int d = 0; d < 3; ++d)
        ext[d] = d < dims(m) ? int64_t(m.owned_cells[d]) + 2 * m.halo_width + (m.entity == 1 ? 0 : 1) : 1;
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

bool stencil_in_range(const Spline3& sd, const int64_t* ext, int nd) {
    for (int d = 0; d < nd; ++d) {
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
        case 4:    // TensorDivergenceP2G (:1544-1555) -> P2G::divergence :712-747
        case 5: {  // the same on the transposed tensor (no reference counterpart)
            double pd[3][3];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) pd[a][b] = mult * (kind == 5 ? xp[b * 3 + a] : xp[a * 3 + b]);
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

// Components per point of each operator kind: scalars 1, vectors nd,
// tensors nd * nd.
int p2g_comps(int kind, int nd = 3) {
    switch (kind) {
        case 0: case 2: return 1;
        case 1: case 3: return nd;
        case 4: case 5: return nd * nd;
    }
    return -1;
}
int g2p_comps(int kind, int nd = 3) {
    switch (kind) {
        case 0: case 4: return 1;
        case 1: case 2: return nd;
        case 3: case 5: return nd * nd;
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
        case 3:    // VectorGradientG2P -> G2P::gradient :247-282 (result[m][n] = d_m W * f_n)
        case 5: {  // the same stored transposed (no reference counterpart)
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
                for (int b = 0; b < 3; ++b) xp[kind == 5 ? b * 3 + a : a * 3 + b] += mult * result[a][b];
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

// P2G:: thread-level operators, 2D specialisations (Interpolation.hpp:
// 466-485, :527-547, :597-621, :674-702, :756-788); the functors premultiply
// as in 3D.
void p2g_point2(int kind, double mult, const double* xp, const Spline3& sd, GridView& v) {
    const int nk = sd.nk;
    switch (kind) {
        case 0: {  // ScalarValueP2G -> P2G::value :466-485
            double pd = xp[0] * mult;
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j) v.at(sd.s[0][i], sd.s[1][j], 0, 0) += pd * sd.w[0][i] * sd.w[1][j];
            return;
        }
        case 1: {  // VectorValueP2G -> P2G::value :527-547
            double pd[2];
            for (int d = 0; d < 2; ++d) pd[d] = mult * xp[d];
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int d = 0; d < 2; ++d) v.at(sd.s[0][i], sd.s[1][j], 0, d) += pd[d] * sd.w[0][i] * sd.w[1][j];
            return;
        }
        case 2: {  // ScalarGradientP2G -> P2G::gradient :597-621
            double pd = xp[0] * mult;
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j) {
                    v.at(sd.s[0][i], sd.s[1][j], 0, 0) += pd * sd.g[0][i] * sd.w[1][j];
                    v.at(sd.s[0][i], sd.s[1][j], 0, 1) += pd * sd.w[0][i] * sd.g[1][j];
                }
            return;
        }
        case 3: {  // VectorDivergenceP2G -> P2G::divergence :674-702
            double pd[2];
            for (int d = 0; d < 2; ++d) pd[d] = mult * xp[d];
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j) {
                    double result = pd[0] * sd.g[0][i] * sd.w[1][j] + pd[1] * sd.w[0][i] * sd.g[1][j];
                    v.at(sd.s[0][i], sd.s[1][j], 0, 0) += result;
                }
            return;
        }
        case 4:    // TensorDivergenceP2G -> P2G::divergence :756-788
        case 5: {  // the same on the transposed tensor
            double pd[2][2];
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b) pd[a][b] = mult * (kind == 5 ? xp[b * 2 + a] : xp[a * 2 + b]);
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j) {
                    double rg[2] = {sd.g[0][i] * sd.w[1][j], sd.w[0][i] * sd.g[1][j]};
                    for (int d1 = 0; d1 < 2; ++d1)
                        for (int d0 = 0; d0 < 2; ++d0) v.at(sd.s[0][i], sd.s[1][j], 0, d0) += rg[d1] * pd[d0][d1];
                }
            return;
        }
    }
}

// G2P:: thread-level operators, 2D specialisations (Interpolation.hpp:81-98,
// :139-158, :212-237, :291-323, :373-396); x += multiplier * result.
void g2p_point2(int kind, double mult, double* xp, const Spline3& sd, GridView& v) {
    const int nk = sd.nk;
    switch (kind) {
        case 0: {  // ScalarValueG2P -> G2P::value :81-98
            double result = 0.0;
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j) result += v.at(sd.s[0][i], sd.s[1][j], 0, 0) * sd.w[0][i] * sd.w[1][j];
            xp[0] += mult * result;
            return;
        }
        case 1: {  // VectorValueG2P -> G2P::value :139-158
            double result[2] = {0.0, 0.0};
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    for (int d = 0; d < 2; ++d)
                        result[d] += v.at(sd.s[0][i], sd.s[1][j], 0, d) * sd.w[0][i] * sd.w[1][j];
            for (int d = 0; d < 2; ++d) xp[d] += mult * result[d];
            return;
        }
        case 2: {  // ScalarGradientG2P -> G2P::gradient :212-237
            double result[2] = {0.0, 0.0};
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j) {
                    double f = v.at(sd.s[0][i], sd.s[1][j], 0, 0);
                    result[0] += f * sd.g[0][i] * sd.w[1][j];
                    result[1] += f * sd.w[0][i] * sd.g[1][j];
                }
            for (int d = 0; d < 2; ++d) xp[d] += mult * result[d];
            return;
        }
        case 3:    // VectorGradientG2P -> G2P::gradient :291-323 (result[m][n] = d_m W * f_n)
        case 5: {  // the same stored transposed
            double result[2][2] = {{0, 0}, {0, 0}};
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j) {
                    double rg[2] = {sd.g[0][i] * sd.w[1][j], sd.w[0][i] * sd.g[1][j]};
                    for (int d0 = 0; d0 < 2; ++d0) {
                        double mg = rg[d0];
                        for (int d1 = 0; d1 < 2; ++d1) result[d0][d1] += mg * v.at(sd.s[0][i], sd.s[1][j], 0, d1);
                    }
                }
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b) xp[kind == 5 ? b * 2 + a : a * 2 + b] += mult * result[a][b];
            return;
        }
        case 4: {  // VectorDivergenceG2P -> G2P::divergence :373-396
            double result = 0.0;
            for (int i = 0; i < nk; ++i)
                for (int j = 0; j < nk; ++j)
                    result += v.at(sd.s[0][i], sd.s[1][j], 0, 0) * sd.g[0][i] * sd.w[1][j] +
                              v.at(sd.s[0][i], sd.s[1][j], 0, 1) * sd.w[0][i] * sd.g[1][j];
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
        if (d >= dims(m)) {  // the single layer of a 2D mesh
            own[d] = idx[d];
            continue;
        }
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
    const int nd = dims(*mesh);
    auto apply = [&](int o, int64_t p, const Spline3& sd, GridView& v) {
        const double* xp = ops[o].x + p * p2g_comps(ops[o].kind, nd);
        if (nd == 2)
            p2g_point2(ops[o].kind, ops[o].multiplier, xp, sd, v);
        else
            p2g_point(ops[o].kind, ops[o].multiplier, xp, sd, v);
    };
    int skipped = 0;
    if (nthreads <= 1) {
        std::vector<GridView> views;
        for (int o = 0; o < n_ops; ++o) views.push_back({ops[o].array, ext[0], ext[1], ext[2], ops[o].dofs});
        for (int64_t p = 0; p < num_point; ++p) {
            Spline3 sd;
            evaluate(*mesh, order, points + nd * p, sd);
            if (!stencil_in_range(sd, ext, nd)) { ++skipped; continue; }
            for (int o = 0; o < n_ops; ++o) apply(o, p, sd, views[o]);
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
                evaluate(*mesh, order, points + nd * p, sd);
                if (!stencil_in_range(sd, ext, nd)) { ++skipped; continue; }
                for (int o = 0; o < n_ops; ++o) apply(o, p, sd, views[o]);
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
    const int nd = dims(*mesh);
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
        evaluate(*mesh, order, points + nd * p, sd);
        if (!stencil_in_range(sd, ext, nd)) { ++skipped; continue; }
        for (int o = 0; o < n_ops; ++o) {
            GridView v = views[o];
            double* xp = ops[o].x + p * g2p_comps(ops[o].kind, nd);
            if (nd == 2)
                g2p_point2(ops[o].kind, ops[o].multiplier, xp, sd, v);
            else
                g2p_point(ops[o].kind, ops[o].multiplier, xp, sd, v);
        }
    }
    return skipped;
}

// Fused g2p2g (the composition of benchmark/grid/
// Cabana_Grid_InterpolationPerformance.cpp:129-174, with G2P reading every
// array as it was at the call): halo.gather on the G2P arrays, then per
// point one spline evaluation, the G2P functors, the P2G functors; then
// halo.scatter(Sum) on the P2G arrays. 3D meshes only (returns -1 otherwise).
int oracle_g2p2g(const oracle_mesh* mesh, const double* points, int64_t num_point, int order,
                 const oracle_op* g2p_ops, int n_g2p, const oracle_op* p2g_ops, int n_p2g) {
    if (dims(*mesh) != 3) return -1;
    int64_t ext[3];
    extents(*mesh, ext);
    const int nd = 3;
    for (int o = 0; o < n_g2p; ++o) {
        bool seen = false;
        for (int q = 0; q < o; ++q) seen |= (g2p_ops[q].array == g2p_ops[o].array);
        if (!seen) oracle_halo_gather(mesh, g2p_ops[o].array, g2p_ops[o].dofs);
    }
    const int64_t nnode = ext[0] * ext[1] * ext[2];
    std::vector<std::vector<double>> snaps(n_g2p);
    std::vector<GridView> gviews, pviews;
    for (int o = 0; o < n_g2p; ++o) {
        double* src = g2p_ops[o].array;
        snaps[o].assign(src, src + nnode * g2p_ops[o].dofs);  // the state at the call
        gviews.push_back({snaps[o].data(), ext[0], ext[1], ext[2], g2p_ops[o].dofs});
    }
    for (int o = 0; o < n_p2g; ++o) pviews.push_back({p2g_ops[o].array, ext[0], ext[1], ext[2], p2g_ops[o].dofs});
    int skipped = 0;
    for (int64_t p = 0; p < num_point; ++p) {
        Spline3 sd;
        evaluate(*mesh, order, points + nd * p, sd);
        if (!stencil_in_range(sd, ext, nd)) { ++skipped; continue; }
        for (int o = 0; o < n_g2p; ++o)
            g2p_point(g2p_ops[o].kind, g2p_ops[o].multiplier, g2p_ops[o].x + p * g2p_comps(g2p_ops[o].kind), sd,
                      gviews[o]);
        for (int o = 0; o < n_p2g; ++o)
            p2g_point(p2g_ops[o].kind, p2g_ops[o].multiplier, p2g_ops[o].x + p * p2g_comps(p2g_ops[o].kind), sd,
                      pviews[o]);
    }
    for (int o = 0; o < n_p2g; ++o) {
        bool seen = false;
        for (int q = 0; q < o; ++q) seen |= (p2g_ops[q].array == p2g_ops[o].array);
        if (!seen) oracle_halo_scatter_sum(mesh, p2g_ops[o].array, p2g_ops[o].dofs);
    }
    return skipped;
}

// CartesianGrid::init, Cabana_CartesianGrid.hpp:61-73 and cellsBetween :279-283.
void oracle_cartesian_num_bins(const double* grid_min, const double* grid_max,
                               const double* grid_delta, int32_t* nbin) {
    for (int d = 0; d < 3; ++d)
        nbin[d] = static_cast<int32_t>(std::floor((grid_max[d] - grid_min[d]) * (1.0 / grid_delta[d])));
}

// LinkedCellList<..., nd>::build, Cabana_LinkedCellList.hpp:652-745, for nd
// = 2 or 3 coordinates per point (positions[nd * p + d]; grid arrays with nd
// entries), run serially so that particles inside a bin keep ascending index
// order.
void oracle_linked_cell_build_nd(int nd, const double* positions, int64_t begin, int64_t end,
                                 const double* grid_min, const double* grid_max,
                                 const double* grid_delta, int32_t* counts, uint64_t* offsets,
                                 uint64_t* permutes) {
    int32_t nx[3] = {1, 1, 1};
    double rdx[3] = {1.0, 1.0, 1.0};
    for (int d = 0; d < nd; ++d) {
        // CartesianGrid::init, Cabana_CartesianGrid.hpp:61-73
        nx[d] = static_cast<int32_t>(std::floor((grid_max[d] - grid_min[d]) * (1.0 / grid_delta[d])));
        const double dx = (grid_max[d] - grid_min[d]) / nx[d];
        rdx[d] = 1.0 / dx;
    }
    const int64_t ncell = int64_t(nx[0]) * nx[1] * nx[2];
    auto cell_of = [&](int64_t p) {
        int c[3] = {0, 0, 0};
        for (int d = 0; d < nd; ++d) {
            // locatePoint, CartesianGrid.hpp:171-182 (2D :158-168)
            c[d] = static_cast<int>(std::floor((positions[nd * p + d] - grid_min[d]) * rdx[d]));
            c[d] = (c[d] == nx[d]) ? c[d] - 1 : c[d];
        }
        // cardinalCellIndex, CartesianGrid.hpp:226-231; in 2D (:233-238)
        // i * nx[1] + j, the same number with nx[2] == 1 and c[2] == 0
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

void oracle_linked_cell_build(const double* positions, int64_t begin, int64_t end,
                              const double* grid_min, const double* grid_max,
                              const double* grid_delta, int32_t* counts, uint64_t* offsets,
                              uint64_t* permutes) {
    oracle_linked_cell_build_nd(3, positions, begin, end, grid_min, grid_max, grid_delta, counts,
                                offsets, permutes);
}

// Cabana::binByKey / sortByKey over int keys (core/src/Cabana_Sort.hpp:217-235
// Impl::kokkosBinSort1d, :364-443). The bin map is Kokkos::BinOp1D, from
// Kokkos (an external dependency of the reference, >= 4.1, not vendored):
// max_bins = nbin + 1, mul = nbin / (max - min) over keys[begin, end), or 1
// for integer keys when max - min <= nbin, bin = int(mul * (key - min)). The
// BinSort order is by bin, then (sort_within_bins) by key; entries that tie
// keep ascending index order (the serial order). counts / offsets: nbin + 1.
void oracle_bin_by_key_range(const int32_t* keys, int64_t begin, int64_t end, int32_t nbin,
                             int sort_within_bins, int32_t* counts, uint64_t* offsets,
                             uint64_t* permutes) {
    const int64_t nbins = int64_t(nbin) + 1;
    std::fill(counts, counts + nbins, 0);
    std::fill(offsets, offsets + nbins, uint64_t(0));
    if (end <= begin) return;
    int32_t kmin = keys[begin], kmax = keys[begin];
    for (int64_t p = begin; p < end; ++p) {
        kmin = std::min(kmin, keys[p]);
        kmax = std::max(kmax, keys[p]);
    }
    const double range = static_cast<double>(kmax) - static_cast<double>(kmin);
    const double mul = range <= static_cast<double>(nbin) ? 1.0 : static_cast<double>(nbin) / range;
    auto bin_of = [&](int64_t p) {
        return static_cast<int>(mul * (static_cast<double>(keys[p]) - static_cast<double>(kmin)));
    };
    for (int64_t p = begin; p < end; ++p) counts[bin_of(p)] += 1;
    uint64_t run = 0;
    for (int64_t b = 0; b < nbins; ++b) {
        offsets[b] = run;
        run += counts[b];
    }
    std::vector<int64_t> order;
    order.reserve(size_t(end - begin));
    for (int64_t p = begin; p < end; ++p) order.push_back(p);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        const int ba = bin_of(a), bb = bin_of(b);
        if (ba != bb) return ba < bb;
        return sort_within_bins ? keys[a] < keys[b] : false;
    });
    for (size_t q = 0; q < order.size(); ++q) permutes[q] = uint64_t(order[q]);
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

void oracle_spline_hessian(int order, double x0, double rdx, double* h) { hessian(order, x0, rdx, h); }

}  // extern "C"

namespace {

// Node weight W_n, its gradient dW[e] and Hessian ddW[e][d] at stencil node
// (i, j, k) of a point, from the per-dimension value / gradient / second
// derivative tables.
struct NodeWeights {
    double W;
    double dW[3];
    double ddW[3][3];
};

NodeWeights node_weights(const Spline3& sd, const double (*h)[kMaxKnot], int i, int j, int k) {
    const int id[3] = {i, j, k};
    NodeWeights nw;
    nw.W = sd.w[0][i] * sd.w[1][j] * sd.w[2][k];
    for (int e = 0; e < 3; ++e) {
        double t = 1.0;
        for (int a = 0; a < 3; ++a) t *= (a == e) ? sd.g[a][id[a]] : sd.w[a][id[a]];
        nw.dW[e] = t;
        for (int d = 0; d < 3; ++d) {
            double u = 1.0;
            for (int a = 0; a < 3; ++a) {
                if (a == e && a == d)
                    u *= h[a][id[a]];
                else if (a == e || a == d)
                    u *= sd.g[a][id[a]];
                else
                    u *= sd.w[a][id[a]];
            }
            nw.ddW[e][d] = u;
        }
    }
    return nw;
}

void halo_apply(const oracle_mesh& m, double* array, int dofs, bool gather_add) {
    int64_t ext[3];
    extents(m, ext);
    GridView v{array, ext[0], ext[1], ext[2], dofs};
    for (int64_t i = 0; i < ext[0]; ++i)
        for (int64_t j = 0; j < ext[1]; ++j)
            for (int64_t k = 0; k < ext[2]; ++k) {
                int64_t idx[3] = {i, j, k}, own[3];
                if (!halo_partner(m, ext, idx, own)) continue;
                for (int c = 0; c < dofs; ++c) {
                    if (gather_add) {
                        v.at(i, j, k, c) += v.at(own[0], own[1], own[2], c);
                    } else {
                        v.at(own[0], own[1], own[2], c) += v.at(i, j, k, c);
                        v.at(i, j, k, c) = 0.0;
                    }
                }
            }
}

}  // namespace

extern "C" {

void oracle_stable_sort_keys(const uint64_t* keys, int64_t n, uint64_t* permutes) {
    std::vector<uint64_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return keys[a] < keys[b]; });
    std::copy(idx.begin(), idx.end(), permutes);
}


// Reverse-mode derivative of oracle_p2g (no reference counterpart): each
// forward operator written out term by term, differentiated by hand with
// respect to its point field and to the point position. array_bar holds
// dL/d(array); on periodic meshes the adjoint of the halo scatter(Sum)
// (ghost += owned image) is applied to it first, in place.
int oracle_p2g_adjoint(const oracle_mesh* mesh, const double* points, int64_t num_point, int order,
                       const oracle_adjoint_op* ops, int n_ops, double* points_bar) {
    if (dims(*mesh) != 3) return -1;  // the adjoints are written for 3D meshes
    int64_t ext[3];
    extents(*mesh, ext);
    const int nd = 3;
    for (int o = 0; o < n_ops; ++o) {
        bool seen = false;
        for (int q = 0; q < o; ++q) seen |= (ops[q].array_bar == ops[o].array_bar);
        if (!seen) halo_apply(*mesh, ops[o].array_bar, ops[o].dofs, true);
    }
    int skipped = 0;
    for (int64_t p = 0; p < num_point; ++p) {
        Spline3 sd;
        evaluate(*mesh, order, points + 3 * p, sd);
        if (!stencil_in_range(sd, ext, nd)) { ++skipped; continue; }
        double h[3][kMaxKnot];
        for (int d = 0; d < 3; ++d) hessian(order, sd.x[d], 1.0 / sd.dx[d], h[d]);
        double pos[3] = {0.0, 0.0, 0.0};
        for (int o = 0; o < n_ops; ++o) {
            const oracle_adjoint_op& op = ops[o];
            const int nc = p2g_comps(op.kind);
            const double* x = op.x ? op.x + p * nc : nullptr;
            double* xb = op.x_bar ? op.x_bar + p * nc : nullptr;
            GridView v{op.array_bar, ext[0], ext[1], ext[2], op.dofs};
            const double m = op.multiplier;
            for (int i = 0; i < sd.nk; ++i)
                for (int j = 0; j < sd.nk; ++j)
                    for (int k = 0; k < sd.nk; ++k) {
                        const NodeWeights nw = node_weights(sd, h, i, j, k);
                        double A[3];
                        for (int c = 0; c < 3; ++c)
                            A[c] = c < op.dofs ? v.at(sd.s[0][i], sd.s[1][j], sd.s[2][k], c) : 0.0;
                        for (int e = 0; e < 3; ++e) {
                            double t = 0.0;
                            switch (op.kind) {
                                case 0: if (x) t = x[0] * A[0] * nw.dW[e]; break;
                                case 1: if (x) for (int d = 0; d < 3; ++d) t += x[d] * A[d] * nw.dW[e]; break;
                                case 2: if (x) for (int d = 0; d < 3; ++d) t += x[0] * A[d] * nw.ddW[e][d]; break;
                                case 3: if (x) for (int d = 0; d < 3; ++d) t += A[0] * x[d] * nw.ddW[e][d]; break;
                                case 4:
                                    if (x) for (int a = 0; a < 3; ++a)
                                        for (int d = 0; d < 3; ++d) t += A[a] * x[a * 3 + d] * nw.ddW[e][d];
                                    break;
                                case 5:
                                    if (x) for (int a = 0; a < 3; ++a)
                                        for (int d = 0; d < 3; ++d) t += A[a] * x[d * 3 + a] * nw.ddW[e][d];
                                    break;
                            }
                            pos[e] += m * t;
                        }
                        if (!xb) continue;
                        switch (op.kind) {
                            case 0: xb[0] += m * A[0] * nw.W; break;
                            case 1: for (int d = 0; d < 3; ++d) xb[d] += m * A[d] * nw.W; break;
                            case 2: for (int d = 0; d < 3; ++d) xb[0] += m * A[d] * nw.dW[d]; break;
                            case 3: for (int d = 0; d < 3; ++d) xb[d] += m * A[0] * nw.dW[d]; break;
                            case 4:
                                for (int a = 0; a < 3; ++a)
                                    for (int d = 0; d < 3; ++d) xb[a * 3 + d] += m * A[a] * nw.dW[d];
                                break;
                            case 5:
                                for (int a = 0; a < 3; ++a)
                                    for (int d = 0; d < 3; ++d) xb[d * 3 + a] += m * A[a] * nw.dW[d];
                                break;
                        }
                    }
        }
        if (points_bar)
            for (int e = 0; e < 3; ++e) points_bar[p * 3 + e] += pos[e];
    }
    return skipped;
}

// Reverse-mode derivative of oracle_g2p (no reference counterpart). x_bar
// holds dL/d(forward output field); array is the forward array as the
// forward read it (after its halo gather). array_bar (may be NULL) receives
// dL/d(array); on periodic meshes the adjoint of the halo gather (owned image
// += ghost, ghost = 0) is applied to it afterwards.
int oracle_g2p_adjoint(const oracle_mesh* mesh, const double* points, int64_t num_point, int order,
                       const oracle_adjoint_op* ops, int n_ops, double* points_bar) {
    if (dims(*mesh) != 3) return -1;  // the adjoints are written for 3D meshes
    int64_t ext[3];
    extents(*mesh, ext);
    const int nd = 3;
    int skipped = 0;
    for (int64_t p = 0; p < num_point; ++p) {
        Spline3 sd;
        evaluate(*mesh, order, points + 3 * p, sd);
        if (!stencil_in_range(sd, ext, nd)) { ++skipped; continue; }
        double h[3][kMaxKnot];
        for (int d = 0; d < 3; ++d) hessian(order, sd.x[d], 1.0 / sd.dx[d], h[d]);
        double pos[3] = {0.0, 0.0, 0.0};
        for (int o = 0; o < n_ops; ++o) {
            const oracle_adjoint_op& op = ops[o];
            const int nc = g2p_comps(op.kind);
            const double* sb = op.x_bar + p * nc;
            GridView va{op.array, ext[0], ext[1], ext[2], op.dofs};
            GridView vb{op.array_bar, ext[0], ext[1], ext[2], op.dofs};
            const double m = op.multiplier;
            for (int i = 0; i < sd.nk; ++i)
                for (int j = 0; j < sd.nk; ++j)
                    for (int k = 0; k < sd.nk; ++k) {
                        const int ni = sd.s[0][i], nj = sd.s[1][j], nkk = sd.s[2][k];
                        const NodeWeights nw = node_weights(sd, h, i, j, k);
                        if (op.array) {
                            double A[3];
                            for (int c = 0; c < 3; ++c) A[c] = c < op.dofs ? va.at(ni, nj, nkk, c) : 0.0;
                            for (int e = 0; e < 3; ++e) {
                                double t = 0.0;
                                switch (op.kind) {
                                    case 0: t = sb[0] * A[0] * nw.dW[e]; break;
                                    case 1: for (int d = 0; d < 3; ++d) t += sb[d] * A[d] * nw.dW[e]; break;
                                    case 2: for (int d = 0; d < 3; ++d) t += sb[d] * A[0] * nw.ddW[e][d]; break;
                                    case 3:
                                        for (int a = 0; a < 3; ++a)
                                            for (int b = 0; b < 3; ++b) t += sb[a * 3 + b] * A[b] * nw.ddW[e][a];
                                        break;
                                    case 4: for (int d = 0; d < 3; ++d) t += sb[0] * A[d] * nw.ddW[e][d]; break;
                                    case 5:
                                        for (int a = 0; a < 3; ++a)
                                            for (int b = 0; b < 3; ++b) t += sb[b * 3 + a] * A[b] * nw.ddW[e][a];
                                        break;
                                }
                                pos[e] += m * t;
                            }
                        }
                        if (!op.array_bar) continue;
                        switch (op.kind) {
                            case 0: vb.at(ni, nj, nkk, 0) += m * sb[0] * nw.W; break;
                            case 1: for (int d = 0; d < 3; ++d) vb.at(ni, nj, nkk, d) += m * sb[d] * nw.W; break;
                            case 2: for (int d = 0; d < 3; ++d) vb.at(ni, nj, nkk, 0) += m * sb[d] * nw.dW[d]; break;
                            case 3:
                                for (int a = 0; a < 3; ++a)
                                    for (int b = 0; b < 3; ++b) vb.at(ni, nj, nkk, b) += m * sb[a * 3 + b] * nw.dW[a];
                                break;
                            case 4: for (int d = 0; d < 3; ++d) vb.at(ni, nj, nkk, d) += m * sb[0] * nw.dW[d]; break;
                            case 5:
                                for (int a = 0; a < 3; ++a)
                                    for (int b = 0; b < 3; ++b) vb.at(ni, nj, nkk, b) += m * sb[b * 3 + a] * nw.dW[a];
                                break;
                        }
                    }
        }
        if (points_bar)
            for (int e = 0; e < 3; ++e) points_bar[p * 3 + e] += pos[e];
    }
    for (int o = 0; o < n_ops; ++o) {
        if (!ops[o].array_bar) continue;
        bool seen = false;
        for (int q = 0; q < o; ++q) seen |= (ops[q].array_bar == ops[o].array_bar);
        if (!seen) halo_apply(*mesh, ops[o].array_bar, ops[o].dofs, false);
    }
    return skipped;
}
}  // extern "C"
