// cgx_cabana.hpp -- C++ shim with the shapes of Cabana::Grid's interpolation
// API over the cgx C ABI (include/cgx.h).
//
// Same names and argument order as the reference
// (grid/src/Cabana_Grid_Interpolation.hpp:831-1566):
//
//   p2g(functor, points, num_point, Spline<N>(), halo, array)
//   g2p(array, halo, points, num_point, Spline<N>(), functor)
//   create{Scalar,Vector}{Value,Gradient,Divergence}{P2G,G2P}, createTensorDivergenceP2G
//
// with light-weight stand-ins for the Kokkos types: `View<T, Rank>` is a
// device pointer with Kokkos LayoutRight strides (or an AoSoA slice), `Array<T>`
// is an (i, j, k, dof) LayoutRight device array over a uniform mesh's ghosted
// nodes (Cabana_Grid_Array.hpp:44-300), `Halo` marks the single-rank halo
// step. A Kokkos build maps Kokkos::View / Cabana::Slice / Grid::Array onto
// these in a few lines (see the field() helpers). Errors become
// std::runtime_error with cgx_last_error(), as the reference throws for host
// misuse. User-defined functors cannot cross the C ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "cgx.h"

namespace cgx {
namespace cabana {

template <int Order>
struct Spline {
    static constexpr int order = Order;
};

struct Node {};
struct NodeHaloPattern {};

inline void check(cgx_status s) {
    if (s != CGX_OK) throw std::runtime_error(std::string("cgx: ") + cgx_last_error());
}

template <class T>
constexpr int32_t dtype_of() {
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value, "float or double fields only");
    return std::is_same<T, double>::value ? CGX_F64 : CGX_F32;
}

// A particle field: element (p, c) at data[(p / vl) * soa_stride + p % vl +
// c * comp_stride]. Rank 1: (p); rank 2: (p, d); rank 3: (p, m, n) with the
// flattened component c = m * 3 + n (Cabana_Slice.hpp:96-190).
template <class T, int Rank>
struct View {
    T* data = nullptr;
    int32_t vector_length = 1;
    int64_t soa_stride = 1;
    int64_t comp_stride = 1;
    static constexpr int rank = Rank;
    using value_type = T;

    // Kokkos LayoutRight (p, ...) with `comps` components per point.
    static View layout_right(T* p, int64_t comps) {
        View v;
        v.data = p;
        v.soa_stride = comps;
        v.comp_stride = 1;
        return v;
    }
    // Kokkos LayoutLeft (p, ...) over n points.
    static View layout_left(T* p, int64_t n) {
        View v;
        v.data = p;
        v.soa_stride = 1;
        v.comp_stride = n;
        return v;
    }
    // Cabana::Slice of an AoSoA member (vector length vl, soa_stride member
    // elements per SoA).
    static View slice(T* p, int32_t vl, int64_t soa) {
        View v;
        v.data = p;
        v.vector_length = vl;
        v.soa_stride = soa;
        v.comp_stride = vl;
        return v;
    }
    cgx_field field() const {
        cgx_field f;
        f.data = data;
        f.dtype = dtype_of<T>();
        f.vector_length = vector_length;
        f.soa_stride = soa_stride;
        f.comp_stride = comp_stride;
        return f;
    }
};

// Uniform local mesh of one rank: what Cabana's LocalGrid / LocalMesh give
// cgx_mesh (ghost low corner, cell size, owned cells, halo width, periodic).
struct LocalMesh {
    cgx_mesh mesh{};
    static LocalMesh uniform(const double low[3], double cell_size, const int32_t owned_cells[3], int halo_width,
                             const bool periodic[3] = nullptr) {
        LocalMesh m;
        for (int d = 0; d < 3; ++d) {
            m.mesh.ghost_low[d] = low[d] - halo_width * cell_size;
            m.mesh.cell_size[d] = cell_size;
            m.mesh.owned_cells[d] = owned_cells[d];
            m.mesh.periodic[d] = periodic ? (periodic[d] ? 1 : 0) : 0;
        }
        m.mesh.halo_width = halo_width;
        m.mesh.entity = CGX_NODE;
        return m;
    }
    int64_t extent(int d) const { return int64_t(mesh.owned_cells[d]) + 2 * mesh.halo_width + 1; }
    int64_t num_nodes() const { return extent(0) * extent(1) * extent(2); }
};

// Grid array over the ghosted nodes, (i, j, k, dof) LayoutRight. It does
// not own `data`: allocate it with cudaMalloc (num_nodes() * dofs elements).
template <class T>
struct Array {
    LocalMesh local_mesh;
    T* data = nullptr;
    int32_t dofs = 1;
    cgx_array array() const {
        cgx_array a;
        a.data = data;
        a.dtype = dtype_of<T>();
        a.dofs = dofs;
        return a;
    }
};

template <class T>
Array<T> createArray(const LocalMesh& m, int dofs, T* device_data) {
    Array<T> a;
    a.local_mesh = m;
    a.data = device_data;
    a.dofs = dofs;
    return a;
}

// Single-rank halo of NodeHaloPattern<3>: periodic folds / fills.
struct Halo {
    int width = 1;
};
inline Halo createHalo(NodeHaloPattern, int width) { return Halo{width}; }

// ArrayOp::assign(array, value, Ghost()) (Cabana_Grid_Array.hpp:431-447).
template <class T>
void assign(const Array<T>& a, double value, void* stream = nullptr) {
    const cgx_array arr = a.array();
    check(cgx_array_assign(&a.local_mesh.mesh, &arr, value, stream));
}

// ---- functors (Cabana_Grid_Interpolation.hpp:938-1566) --------------------

template <class ViewT, int Kind, bool IsP2G>
struct Functor {
    ViewT x;
    double multiplier;
    static constexpr int kind = Kind;
    static constexpr bool is_p2g = IsP2G;
};

template <class V> using ScalarValueP2G = Functor<V, CGX_SCALAR_VALUE_P2G, true>;
template <class V> using VectorValueP2G = Functor<V, CGX_VECTOR_VALUE_P2G, true>;
template <class V> using ScalarGradientP2G = Functor<V, CGX_SCALAR_GRADIENT_P2G, true>;
template <class V> using VectorDivergenceP2G = Functor<V, CGX_VECTOR_DIVERGENCE_P2G, true>;
template <class V> using TensorDivergenceP2G = Functor<V, CGX_TENSOR_DIVERGENCE_P2G, true>;
template <class V> using ScalarValueG2P = Functor<V, CGX_SCALAR_VALUE_G2P, false>;
template <class V> using VectorValueG2P = Functor<V, CGX_VECTOR_VALUE_G2P, false>;
template <class V> using ScalarGradientG2P = Functor<V, CGX_SCALAR_GRADIENT_G2P, false>;
template <class V> using VectorGradientG2P = Functor<V, CGX_VECTOR_GRADIENT_G2P, false>;
template <class V> using VectorDivergenceG2P = Functor<V, CGX_VECTOR_DIVERGENCE_G2P, false>;

// The factories check the field rank at compile time, as the reference's
// functors static_assert it.
#define CGX_FACTORY(NAME, RANK)                                                   \
    template <class V>                                                            \
    NAME<V> create##NAME(const V& x, double multiplier) {                         \
        static_assert(V::rank == RANK, #NAME " needs a rank-" #RANK " field");  \
        return NAME<V>{x, multiplier};                                            \
    }
CGX_FACTORY(ScalarValueP2G, 1)
CGX_FACTORY(VectorValueP2G, 2)
CGX_FACTORY(ScalarGradientP2G, 1)
CGX_FACTORY(VectorDivergenceP2G, 2)
CGX_FACTORY(TensorDivergenceP2G, 3)
CGX_FACTORY(ScalarValueG2P, 1)
CGX_FACTORY(VectorValueG2P, 2)
CGX_FACTORY(ScalarGradientG2P, 2)
CGX_FACTORY(VectorGradientG2P, 3)
CGX_FACTORY(VectorDivergenceG2P, 1)
#undef CGX_FACTORY

// ---- drivers ---------------------------------------------------------------

// Beyond the reference signature: the precision form, an optional tile
// ordering (cgx_sort_tiles) and the stream.
struct Options {
    int precision = CGX_PLAIN_FP64;
    const cgx_tiling* tiling = nullptr;
    void* stream = nullptr;
    unsigned flags = 0;
};

// One handle (workspace, error flag) per host thread.
inline cgx_handle thread_handle() {
    struct Owner {
        cgx_handle h = nullptr;
        Owner() { check(cgx_create(&h)); }
        ~Owner() { cgx_destroy(h); }
    };
    thread_local Owner owner;
    return owner.h;
}

template <class F, class T>
cgx_op make_op(const F& f, const Array<T>& a) {
    cgx_op op{};
    op.kind = F::kind;
    op.multiplier = f.multiplier;
    op.x = f.x.field();
    op.array = a.array();
    return op;
}

// Cabana::Grid::p2g (Interpolation.hpp:1217-1313): adds into `array`, then
// the halo scatter(Sum) when a halo is given.
template <class F, class Points, int N, class T>
void p2g(const F& functor, const Points& points, std::size_t num_point, Spline<N>, const Halo* halo, Array<T>& array,
         const Options& opt = Options()) {
    static_assert(F::is_p2g, "p2g needs a P2G functor");
    const cgx_op op = make_op(functor, array);
    const cgx_field pts = points.field();
    const unsigned fl = opt.flags | (halo ? 0u : CGX_FLAG_SKIP_HALO);
    check(cgx_p2g(thread_handle(), &array.local_mesh.mesh, &pts, int64_t(num_point), N, &op, 1, opt.precision,
                  opt.tiling, fl, opt.stream));
}

template <class F, class Points, int N, class T>
void p2g(const F& functor, const Points& points, std::size_t num_point, Spline<N> s, const Halo& halo,
         Array<T>& array, const Options& opt = Options()) {
    p2g(functor, points, num_point, s, &halo, array, opt);
}

// Cabana::Grid::g2p (Interpolation.hpp:831-927): the halo gather first
// when a halo is given, then x += multiplier * result.
template <class T, class Points, int N, class F>
void g2p(const Array<T>& array, const Halo* halo, const Points& points, std::size_t num_point, Spline<N>,
         const F& functor, const Options& opt = Options()) {
    static_assert(!F::is_p2g, "g2p needs a G2P functor");
    const cgx_op op = make_op(functor, array);
    const cgx_field pts = points.field();
    const unsigned fl = opt.flags | (halo ? 0u : CGX_FLAG_SKIP_HALO);
    check(cgx_g2p(thread_handle(), &array.local_mesh.mesh, &pts, int64_t(num_point), N, &op, 1, opt.precision,
                  opt.tiling, fl, opt.stream));
}

template <class T, class Points, int N, class F>
void g2p(const Array<T>& array, const Halo& halo, const Points& points, std::size_t num_point, Spline<N> s,
         const F& functor, const Options& opt = Options()) {
    g2p(array, &halo, points, num_point, s, functor, opt);
}

}  // namespace cabana
}  // namespace cgx
