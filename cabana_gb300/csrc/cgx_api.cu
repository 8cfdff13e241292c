// C ABI of libcgx: argument checks, workspace, dispatch to the kernels.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cgx_kernels.cuh"

using namespace cgx;

struct cgx_context {
    int device = 0;
    int sms = 0;
    void* ws = nullptr;  // grow-only workspace
    size_t ws_bytes = 0;
    int* flags = nullptr;  // [0] error flag, [1] work counter, [2..3] work count (int64)
    WorkItem* work = nullptr;
    size_t work_cap = 0;
    int64_t* work_prefix = nullptr;
    size_t prefix_cap = 0;
    void* adj = nullptr;  // grow-only: gradient sums of the position adjoint
    size_t adj_bytes = 0;
    int last_dispatch = CGX_DISPATCH_NONE;
};

namespace {

thread_local std::string g_last_error;

cgx_status fail(cgx_status code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

cgx_status cuda_fail(cudaError_t e, const char* where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return CGX_ERR_CUDA;
}

#define CGX_CUDA(call)                                  \
    do {                                                \
        cudaError_t _e = (call);                        \
        if (_e != cudaSuccess) return cuda_fail(_e, #call); \
    } while (0)

cgx_status ensure_ws(cgx_context* h, size_t bytes) {
    if (bytes <= h->ws_bytes) return CGX_OK;
    if (h->ws) cudaFree(h->ws);
    h->ws = nullptr;
    h->ws_bytes = 0;
    size_t want = bytes + bytes / 8 + (1 << 20);
    cudaError_t e = cudaMalloc(&h->ws, want);
    if (e != cudaSuccess) return fail(CGX_ERR_NO_MEMORY, std::string("workspace allocation failed: ") + cudaGetErrorString(e));
    h->ws_bytes = want;
    return CGX_OK;
}

bool valid_dtype(int t) { return t == CGX_F32 || t == CGX_F64; }

// Space dimensions of a mesh (num_space_dim 0 reads as 3).
int mesh_dims(const cgx_mesh& m) { return m.num_space_dim == 2 ? 2 : 3; }

cgx_status check_mesh(const cgx_mesh* m) {
    if (!m) return fail(CGX_ERR_INVALID_ARG, "mesh is NULL");
    if (m->num_space_dim != 0 && m->num_space_dim != 2 && m->num_space_dim != 3)
        return fail(CGX_ERR_INVALID_ARG, "num_space_dim must be 2 or 3");
    const int nd = mesh_dims(*m);
    for (int d = 0; d < nd; ++d) {
        if (!(m->cell_size[d] > 0.0)) return fail(CGX_ERR_INVALID_ARG, "cell_size must be positive");
        if (m->owned_cells[d] < 1) return fail(CGX_ERR_INVALID_ARG, "owned_cells must be >= 1");
    }
    if (m->halo_width < 0) return fail(CGX_ERR_INVALID_ARG, "halo_width must be >= 0");
    if (m->entity != CGX_NODE && m->entity != CGX_CELL) return fail(CGX_ERR_INVALID_ARG, "entity must be CGX_NODE or CGX_CELL");
    for (int d = 0; d < nd; ++d) {
        if (m->periodic[d] && m->halo_width >= m->owned_cells[d])
            return fail(CGX_ERR_INVALID_ARG, "periodic halo wider than the owned cells");
    }
    return CGX_OK;
}

cgx_status check_field(const cgx_field* f, const char* what) {
    if (!f) return fail(CGX_ERR_INVALID_ARG, std::string(what) + " is NULL");
    if (!f->data) return fail(CGX_ERR_INVALID_ARG, std::string(what) + ".data is NULL");
    if (!valid_dtype(f->dtype)) return fail(CGX_ERR_INVALID_ARG, std::string(what) + ": dtype must be CGX_F32 or CGX_F64");
    const int vl = f->vector_length;
    if (vl < 1 || (vl & (vl - 1))) return fail(CGX_ERR_INVALID_ARG, std::string(what) + ": vector_length must be a power of two");
    return CGX_OK;
}

DField to_dfield(const cgx_field& f) {
    DField d;
    d.data = reinterpret_cast<char*>(f.data);
    d.dtype = f.dtype;
    d.log2vl = log2_int(f.vector_length);
    d.soa_stride = f.soa_stride;
    d.comp_stride = f.comp_stride;
    return d;
}

// LocalMesh::coordinates(Entity, index) (grid/src/Cabana_Grid_LocalMesh.hpp:
// 180-200) and the dx / rdx of evaluateSpline (Splines.hpp:1293-1311).
// A 2D mesh has one entity layer in the third dimension (ext 1), so its
// (i, j, dof) arrays index as (i, j, 0, dof).
DMesh to_dmesh(const cgx_mesh& m) {
    DMesh d;
    for (int a = 0; a < 3; ++a) {
        if (a >= mesh_dims(m)) {
            d.low[a] = 0.0;
            d.rdx[a] = 1.0;
            d.rdx_f[a] = 1.0f;
            d.ext[a] = 1;
            continue;
        }
        double lo, hi;
        if (m.entity == CGX_CELL) {
            lo = m.ghost_low[a] + (double(0) + double(0.5)) * m.cell_size[a];
            hi = m.ghost_low[a] + (double(1) + double(0.5)) * m.cell_size[a];
        } else {
            lo = m.ghost_low[a] + double(0) * m.cell_size[a];
            hi = m.ghost_low[a] + double(1) * m.cell_size[a];
        }
        const double dx = hi - lo;
        d.low[a] = lo;
        d.rdx[a] = 1.0 / dx;
        d.rdx_f[a] = float(d.rdx[a]);
        d.ext[a] = m.owned_cells[a] + 2 * m.halo_width + (m.entity == CGX_NODE ? 1 : 0);
    }
    return d;
}

// Point components and array dofs of each operator kind in nd space
// dimensions: scalars 1, vectors nd, tensors nd * nd.
int p2g_comps(int kind, int nd = 3) {
    switch (kind) {
        case CGX_SCALAR_VALUE_P2G: case CGX_SCALAR_GRADIENT_P2G: return 1;
        case CGX_VECTOR_VALUE_P2G: case CGX_VECTOR_DIVERGENCE_P2G: return nd;
        case CGX_TENSOR_DIVERGENCE_P2G: case CGX_TENSOR_DIVERGENCE_T_P2G: return nd * nd;
    }
    return -1;
}
int p2g_dofs(int kind, int nd = 3) {
    switch (kind) {
        case CGX_SCALAR_VALUE_P2G: case CGX_VECTOR_DIVERGENCE_P2G: return 1;
        case CGX_VECTOR_VALUE_P2G: case CGX_SCALAR_GRADIENT_P2G: case CGX_TENSOR_DIVERGENCE_P2G:
        case CGX_TENSOR_DIVERGENCE_T_P2G: return nd;
    }
    return -1;
}
int g2p_comps(int kind, int nd = 3) {
    switch (kind) {
        case CGX_SCALAR_VALUE_G2P: case CGX_VECTOR_DIVERGENCE_G2P: return 1;
        case CGX_VECTOR_VALUE_G2P: case CGX_SCALAR_GRADIENT_G2P: return nd;
        case CGX_VECTOR_GRADIENT_G2P: case CGX_VECTOR_GRADIENT_T_G2P: return nd * nd;
    }
    return -1;
}
int g2p_dofs(int kind, int nd = 3) {
    switch (kind) {
        case CGX_SCALAR_VALUE_G2P: case CGX_SCALAR_GRADIENT_G2P: return 1;
        case CGX_VECTOR_VALUE_G2P: case CGX_VECTOR_GRADIENT_G2P: case CGX_VECTOR_DIVERGENCE_G2P:
        case CGX_VECTOR_GRADIENT_T_G2P: return nd;
    }
    return -1;
}

bool any_periodic(const cgx_mesh& m) {
    bool any = false;
    for (int d = 0; d < mesh_dims(m); ++d) any |= m.periodic[d] != 0;
    return any;
}

HaloParams to_halo(const cgx_mesh& m, const cgx_array& a) {
    HaloParams h;
    h.data = reinterpret_cast<char*>(a.data);
    h.dtype = a.dtype;
    h.dofs = a.dofs;
    h.dims = mesh_dims(m);
    h.reserved = 0;
    for (int d = 0; d < 3; ++d) {
        const bool in = d < h.dims;
        h.ext[d] = in ? m.owned_cells[d] + 2 * m.halo_width + (m.entity == CGX_NODE ? 1 : 0) : 1;
        h.owned_cells[d] = in ? m.owned_cells[d] : 1;
        h.periodic[d] = in && m.periodic[d] ? 1 : 0;
    }
    h.halo_width = m.halo_width;
    h.node_extra = m.entity == CGX_NODE ? 1 : 0;
    return h;
}

cgx_status check_ops(const cgx_op* ops, int n_ops, bool p2g, bool have_points, int nd = 3) {
    if (!ops || n_ops < 1 || n_ops > kMaxOps) return fail(CGX_ERR_INVALID_ARG, "n_ops must be in [1, 8]");
    for (int o = 0; o < n_ops; ++o) {
        const cgx_op& op = ops[o];
        const int comps = p2g ? p2g_comps(op.kind, nd) : g2p_comps(op.kind, nd);
        const int dofs = p2g ? p2g_dofs(op.kind, nd) : g2p_dofs(op.kind, nd);
        if (comps < 0) return fail(CGX_ERR_INVALID_ARG, "unknown operator kind");
        if (have_points) {
            cgx_status s = check_field(&op.x, "op.x");
            if (s) return s;
        }
        if (!op.array.data) return fail(CGX_ERR_INVALID_ARG, "op.array.data is NULL");
        if (!valid_dtype(op.array.dtype)) return fail(CGX_ERR_INVALID_ARG, "op.array.dtype must be CGX_F32 or CGX_F64");
        if (op.array.dofs < dofs) return fail(CGX_ERR_INVALID_ARG, "array has fewer dofs than the operator writes/reads");
    }
    return CGX_OK;
}

cgx_status finish_check(cgx_context* h, unsigned flags, cudaStream_t st) {
    if (!(flags & CGX_FLAG_CHECK_BOUNDS)) return CGX_OK;
    int host_flag = 0;
    CGX_CUDA(cudaMemcpyAsync(&host_flag, h->flags, sizeof(int), cudaMemcpyDeviceToHost, st));
    CGX_CUDA(cudaStreamSynchronize(st));
    if (host_flag & (1 << CGX_ERR_OUT_OF_BOUNDS))
        return fail(CGX_ERR_OUT_OF_BOUNDS, "a point's stencil left the ghosted index space; it was skipped");
    if (host_flag & (1 << CGX_ERR_INVALID_ARG)) return fail(CGX_ERR_INVALID_ARG, "a key was outside [0, nbin)");
    if (host_flag & (1 << CGX_ERR_TIMEOUT))
        return fail(CGX_ERR_TIMEOUT, "a bounded device wait gave up; the results are incomplete");
    return CGX_OK;
}

cgx_status halo_all(const cgx_mesh& m, const cgx_op* ops, int n_ops, int mode, int sms, cudaStream_t st) {
    if (!any_periodic(m)) return CGX_OK;
    for (int o = 0; o < n_ops; ++o) {
        bool seen = false;
        for (int q = 0; q < o; ++q) seen |= ops[q].array.data == ops[o].array.data;
        if (seen) continue;
        CGX_CUDA(launch_halo(to_halo(m, ops[o].array), mode, sms, st));
    }
    return CGX_OK;
}

// Lower the P2G functors to accumulation channels (one grid dof each) and
// group them for the tiled kernel. Value channels receive a * W, gradient
// channels b . grad W (Interpolation.hpp:437-747):
//   ScalarValueP2G      -> 1 value channel      a = m f
//   VectorValueP2G      -> 3 value channels     a = m f_d
//   ScalarGradientP2G   -> 3 gradient channels  b = m f e_d
//   VectorDivergenceP2G -> 1 gradient channel   b = m f
//   TensorDivergenceP2G -> 3 gradient channels  b = m f_{d,:}
//   (transposed form)   -> 3 gradient channels  b = m f_{:,d}
bool plan_channels(TiledParams& prm, const cgx_op* ops, int n_ops, int order) {
    Channel val[kMaxChannels], grd[kMaxChannels];
    int nv = 0, ng = 0;
    int nsrc = 0;
    bool too_many = false;
    auto source = [&](int op, int comp) -> int8_t {
        if (comp < 0) return -1;
        for (int s = 0; s < nsrc; ++s)
            if (prm.sources[s].op == op && prm.sources[s].comp == comp) return int8_t(s);
        if (nsrc == kMaxSources) {
            too_many = true;
            return -1;
        }
        prm.sources[nsrc].op = int8_t(op);
        prm.sources[nsrc].comp = int8_t(comp);
        prm.sources[nsrc].reserved = 0;
        prm.sources[nsrc].mult = float(prm.ops[op].mult);
        return int8_t(nsrc++);
    };
    auto add = [&](bool gradient, int slot, int dof, int op, const int* comps) {
        Channel c;
        c.slot = int8_t(slot);
        c.dof = int8_t(dof);
        for (int n = 0; n < 3; ++n) {
            c.src[n] = source(op, comps[n]);
            c.reserved[n] = 0;
        }
        if (gradient)
            grd[ng++] = c;
        else
            val[nv++] = c;
    };
    for (int o = 0; o < n_ops; ++o) {
        const int slot = prm.ops[o].slot;
        switch (ops[o].kind) {
            case CGX_SCALAR_VALUE_P2G: {
                const int c[3] = {0, -1, -1};
                add(false, slot, 0, o, c);
                break;
            }
            case CGX_VECTOR_VALUE_P2G:
                for (int d = 0; d < 3; ++d) {
                    const int c[3] = {d, -1, -1};
                    add(false, slot, d, o, c);
                }
                break;
            case CGX_SCALAR_GRADIENT_P2G:
                for (int d = 0; d < 3; ++d) {
                    const int c[3] = {d == 0 ? 0 : -1, d == 1 ? 0 : -1, d == 2 ? 0 : -1};
                    add(true, slot, d, o, c);
                }
                break;
            case CGX_VECTOR_DIVERGENCE_P2G: {
                const int c[3] = {0, 1, 2};
                add(true, slot, 0, o, c);
                break;
            }
            case CGX_TENSOR_DIVERGENCE_P2G:
                for (int m = 0; m < 3; ++m) {
                    const int c[3] = {3 * m, 3 * m + 1, 3 * m + 2};
                    add(true, slot, m, o, c);
                }
                break;
            case CGX_TENSOR_DIVERGENCE_T_P2G:
                for (int m = 0; m < 3; ++m) {
                    const int c[3] = {m, 3 + m, 6 + m};
                    add(true, slot, m, o, c);
                }
                break;
        }
    }
    const int cv = p2g_group_capacity(order, false), cg = p2g_group_capacity(order, true);
    int n = 0, g = 0;
    for (int i = 0; i < nv; i += cv) {
        if (g >= kMaxGroups) return false;
        prm.groups[g].gradient = 0;
        prm.groups[g].first = int8_t(n + i);
        prm.groups[g].count = int8_t(nv - i < cv ? nv - i : cv);
        ++g;
    }
    for (int i = 0; i < nv; ++i) prm.channels[n++] = val[i];
    for (int i = 0; i < ng; i += cg) {
        if (g >= kMaxGroups) return false;
        prm.groups[g].gradient = 1;
        prm.groups[g].first = int8_t(n + i);
        prm.groups[g].count = int8_t(ng - i < cg ? ng - i : cg);
        ++g;
    }
    for (int i = 0; i < ng; ++i) prm.channels[n++] = grd[i];
    if (too_many) return false;
    prm.n_sources = nsrc;
    prm.n_channels = n;
    prm.n_groups = g;
    return true;
}

const int64_t kChunk = p2g_tiled_chunk();  // largest work item of the tiled kernels

// Particles per work item for one call: large items flush the node box less
// often, small ones balance small problems; aim for >= 4 items per SM.
int64_t item_particles(const cgx_context* h, int64_t num_point) {
    const int64_t want = num_point / (int64_t(h->sms) * 4);
    int64_t item = 2048;
    while (item < want && item < kChunk) item *= 2;
    return item;
}

cgx_status build_work(cgx_context* h, const cgx_tiling& t, int64_t num_point, cudaStream_t st) {
    const int64_t nt = int64_t(t.num_tiles[0]) * t.num_tiles[1] * t.num_tiles[2];
    const int64_t item = item_particles(h, num_point);
    const size_t cap = size_t(nt + num_point / item + 1);
    if (cap > h->work_cap) {
        if (h->work) cudaFree(h->work);
        h->work = nullptr;
        h->work_cap = 0;
        CGX_CUDA(cudaMalloc(&h->work, cap * sizeof(WorkItem)));
        h->work_cap = cap;
    }
    if (size_t(nt) > h->prefix_cap) {
        if (h->work_prefix) cudaFree(h->work_prefix);
        h->work_prefix = nullptr;
        h->prefix_cap = 0;
        CGX_CUDA(cudaMalloc(&h->work_prefix, size_t(nt) * sizeof(int64_t)));
        h->prefix_cap = size_t(nt);
    }
    cgx_status s = ensure_ws(h, size_t(nt) * 4 + 512 + scan_scratch_bytes(nt));
    if (s) return s;
    CGX_CUDA(build_work_items(t.tile_offsets, nt, item, h->work_prefix, h->work,
                              reinterpret_cast<int64_t*>(h->flags + 2), h->ws, st, h->sms));
    return CGX_OK;
}

// The operator structure of a tiled launch (shared by every instance of a
// batched launch): distinct-array slots, box layout in shared memory, p2g
// channel plan. Returns false when the tiled kernels cannot take it (too
// many channel groups, or node boxes plus staging beyond shared memory).
bool setup_tiled(TiledParams& prm, const cgx_op* ops, int n_ops, int spline_order, bool p2g) {
    std::memset(&prm, 0, sizeof(prm));
    prm.n_ops = n_ops;
    const int nk = spline_order + 1;
    for (int d = 0; d < 3; ++d) {
        prm.tile[d] = kTiledTile;
        prm.box[d] = kTiledTile + nk - 1;
    }
    prm.box_nodes = prm.box[0] * prm.box[1] * prm.box[2];
    int n_arrays = 0;
    int offset = 0;
    for (int o = 0; o < n_ops; ++o) {
        int slot = -1;
        for (int a = 0; a < n_arrays; ++a)
            if (prm.arrays[a].a.data == ops[o].array.data) slot = a;
        if (slot < 0) {
            slot = n_arrays++;
            prm.arrays[slot].a.data = reinterpret_cast<char*>(ops[o].array.data);
            prm.arrays[slot].a.dtype = ops[o].array.dtype;
            prm.arrays[slot].a.dofs = ops[o].array.dofs;
            prm.arrays[slot].smem_offset = offset;
            offset += prm.box_nodes * ops[o].array.dofs * (p2g ? 2 : 1);
        }
        prm.ops[o].kind = ops[o].kind;
        prm.ops[o].slot = slot;
        prm.ops[o].mult = ops[o].multiplier;
        prm.ops[o].mult_f = float(ops[o].multiplier);
    }
    prm.n_arrays = n_arrays;
    prm.smem_floats = offset;
    bool ok = true;
    if (p2g && !plan_channels(prm, ops, n_ops, spline_order)) ok = false;  // too many channel groups
    // node boxes plus per-item staging must fit in one SM's shared memory
    if (p2g) {
        if (p2g_tiled_smem(prm, size_t(offset) * sizeof(float)) > p2g_tiled_smem_limit(spline_order)) ok = false;
    } else {
        // g2p_tiled_smem also refuses double point fields
        for (int o = 0; o < n_ops; ++o) prm.ops[o].x.dtype = ops[o].x.dtype;
        for (int a = 0; a < n_arrays; ++a)
            if (g2p_tiled_smem(prm, a) > 220 * 1024) ok = false;
    }
    return ok;
}

// The mesh and buffers of one instance, with the slots of `prm`. Returns
// false when the mesh is beyond the integer mapping of the tiled kernels
// (origin more than 2^28 cells from zero, or extents of 2^28 nodes).
bool fill_geom(TiledGeom& g, const TiledParams& prm, const cgx_mesh& mesh, const cgx_field& points, const cgx_op* ops,
               int n_ops, const cgx_tiling& tiling, int spline_order) {
    std::memset(&g, 0, sizeof(g));
    g.mesh = to_dmesh(mesh);
    const int shift_even = (spline_order % 2 == 0) ? 1 : 0;
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
        g.c0[d] = -g.mesh.low[d] * g.mesh.rdx[d] + 0.5 * shift_even;
        g.fx[d] = fixed_map(g.mesh.rdx[d], g.c0[d]);
        ok &= fixed_map_ok(g.c0[d]) && g.mesh.ext[d] < (1 << 28);
        g.num_tiles[d] = tiling.num_tiles[d];
    }
    g.points = to_dfield(points);
    for (int o = 0; o < n_ops; ++o) {
        g.x[o] = to_dfield(ops[o].x);
        DArray& a = g.arr[prm.ops[o].slot];
        a.data = reinterpret_cast<char*>(ops[o].array.data);
        a.dtype = ops[o].array.dtype;
        a.dofs = ops[o].array.dofs;
    }
    return ok;
}

cgx_status interpolate(cgx_handle h, const cgx_mesh* mesh, const cgx_field* points, int64_t num_point,
                       int spline_order, const cgx_op* ops, int n_ops, int precision, const cgx_tiling* tiling,
                       unsigned flags, void* stream, bool p2g) {
    if (!h) return fail(CGX_ERR_INVALID_ARG, "handle is NULL");
    cgx_status s = check_mesh(mesh);
    if (s) return s;
    if (num_point < 0) return fail(CGX_ERR_INVALID_ARG, "num_point must be >= 0");
    if (num_point > 0) {
        s = check_field(points, "points");
        if (s) return s;
        if (points->dtype != CGX_F64) return fail(CGX_ERR_INVALID_ARG, "point coordinates must be double (CGX_F64)");
    }
    if (spline_order < 0 || spline_order > 6) return fail(CGX_ERR_NOT_SUPPORTED, "spline order must be in [0, 6]");
    if (precision != CGX_PLAIN_FP64 && precision != CGX_FP32_COMPENSATED)
        return fail(CGX_ERR_INVALID_ARG, "unknown precision");
    const int nd = mesh_dims(*mesh);
    s = check_ops(ops, n_ops, p2g, num_point > 0, nd);
    if (s) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (flags & CGX_FLAG_CHECK_BOUNDS) CGX_CUDA(cudaMemsetAsync(h->flags, 0, sizeof(int), st));

    const DMesh dm = to_dmesh(*mesh);
    if (!p2g && !(flags & CGX_FLAG_SKIP_HALO)) {
        s = halo_all(*mesh, ops, n_ops, kHaloGather, h->sms, st);
        if (s) return s;
    }

    // The tiled kernels are built for cubic tiles of kTiledTile base nodes;
    // other tilings still order the particles but run the point kernels.
    bool tiled = nd == 3 && num_point > 0 && tiling && precision == CGX_FP32_COMPENSATED && tiling->tile_offsets &&
                 tiling->spline_order == spline_order && spline_order >= 1 && spline_order <= 3 &&
                 tiling->tile[0] == kTiledTile && tiling->tile[1] == kTiledTile && tiling->tile[2] == kTiledTile;
    if (tiled) {
        TiledParams prm;
        tiled = setup_tiled(prm, ops, n_ops, spline_order, p2g);
        tiled &= fill_geom(prm.geom, prm, *mesh, *points, ops, n_ops, *tiling, spline_order);
        prm.num_point = num_point;
        const int n_arrays = prm.n_arrays;
        const size_t smem = size_t(prm.smem_floats) * sizeof(float);
        if (tiled) {
            s = build_work(h, *tiling, num_point, st);
            if (s) return s;
            prm.work = h->work;
            prm.work_count = reinterpret_cast<const int64_t*>(h->flags + 2);
            prm.work_counter = h->flags + 1;
            prm.error_flag = h->flags;
            if (p2g) {
                CGX_CUDA(cudaMemsetAsync(h->flags + 1, 0, sizeof(int), st));
                CGX_CUDA(launch_p2g_tiled(prm, spline_order, h->sms, smem, st));
            } else {
                // one launch per source array, its box at shared offset 0
                for (int a = 0; a < n_arrays; ++a) {
                    TiledParams one = prm;
                    one.arrays[a].smem_offset = 0;
                    const size_t smem_a = g2p_tiled_smem(prm, a);
                    CGX_CUDA(cudaMemsetAsync(h->flags + 1, 0, sizeof(int), st));
                    CGX_CUDA(launch_g2p_tiled(one, spline_order, a, h->sms, smem_a, st));
                }
            }
            h->last_dispatch = CGX_DISPATCH_TILED;
        }
    }
    if (!tiled && num_point > 0) {
        PointParams prm;
        std::memset(&prm, 0, sizeof(prm));
        prm.mesh = dm;
        prm.points = to_dfield(*points);
        prm.num_point = num_point;
        prm.n_ops = n_ops;
        prm.dims = nd;
        prm.error_flag = h->flags;
        for (int o = 0; o < n_ops; ++o) {
            prm.ops[o].kind = ops[o].kind;
            prm.ops[o].slot = o;
            prm.ops[o].mult = ops[o].multiplier;
            prm.ops[o].mult_f = float(ops[o].multiplier);
            prm.ops[o].x = to_dfield(ops[o].x);
            prm.ops[o].a.data = reinterpret_cast<char*>(ops[o].array.data);
            prm.ops[o].a.dtype = ops[o].array.dtype;
            prm.ops[o].a.dofs = ops[o].array.dofs;
        }
        CGX_CUDA(launch_points(prm, spline_order, p2g, precision == CGX_PLAIN_FP64, h->sms, st));
        h->last_dispatch = CGX_DISPATCH_POINTS;
    }
    if (p2g && !(flags & CGX_FLAG_SKIP_HALO)) {
        s = halo_all(*mesh, ops, n_ops, kHaloScatterSum, h->sms, st);
        if (s) return s;
    }
    return finish_check(h, flags, st);
}

// Pairing of point field and grid array in the position adjoint of a
// forward operator (see cgx_adjoint.cu); -1 for an unknown kind.
int adjoint_pattern(int kind, bool p2g) {
    if (p2g) {
        switch (kind) {
            case CGX_SCALAR_VALUE_P2G: return kAdjValue1;
            case CGX_VECTOR_VALUE_P2G: return kAdjValue3;
            case CGX_SCALAR_GRADIENT_P2G: return kAdjGradA;
            case CGX_VECTOR_DIVERGENCE_P2G: return kAdjGradS;
            case CGX_TENSOR_DIVERGENCE_P2G: return kAdjTensor;
            case CGX_TENSOR_DIVERGENCE_T_P2G: return kAdjTensorT;
        }
    } else {
        switch (kind) {
            case CGX_SCALAR_VALUE_G2P: return kAdjValue1;
            case CGX_VECTOR_VALUE_G2P: return kAdjValue3;
            case CGX_SCALAR_GRADIENT_G2P: return kAdjGradS;
            case CGX_VECTOR_GRADIENT_G2P: return kAdjTensorT;
            case CGX_VECTOR_DIVERGENCE_G2P: return kAdjGradA;
            case CGX_VECTOR_GRADIENT_T_G2P: return kAdjTensor;
        }
    }
    return -1;
}

// The operator of the other direction whose linear map is the transpose of
// a forward operator's (same multiplier): the value part of its adjoint.
int transpose_kind(int kind, bool p2g) {
    if (p2g) {
        switch (kind) {
            case CGX_SCALAR_VALUE_P2G: return CGX_SCALAR_VALUE_G2P;
            case CGX_VECTOR_VALUE_P2G: return CGX_VECTOR_VALUE_G2P;
            case CGX_SCALAR_GRADIENT_P2G: return CGX_VECTOR_DIVERGENCE_G2P;
            case CGX_VECTOR_DIVERGENCE_P2G: return CGX_SCALAR_GRADIENT_G2P;
            case CGX_TENSOR_DIVERGENCE_P2G: return CGX_VECTOR_GRADIENT_T_G2P;
            case CGX_TENSOR_DIVERGENCE_T_P2G: return CGX_VECTOR_GRADIENT_G2P;
        }
    } else {
        switch (kind) {
            case CGX_SCALAR_VALUE_G2P: return CGX_SCALAR_VALUE_P2G;
            case CGX_VECTOR_VALUE_G2P: return CGX_VECTOR_VALUE_P2G;
            case CGX_SCALAR_GRADIENT_G2P: return CGX_VECTOR_DIVERGENCE_P2G;
            case CGX_VECTOR_GRADIENT_G2P: return CGX_TENSOR_DIVERGENCE_T_P2G;
            case CGX_VECTOR_DIVERGENCE_G2P: return CGX_SCALAR_GRADIENT_P2G;
            case CGX_VECTOR_GRADIENT_T_G2P: return CGX_TENSOR_DIVERGENCE_P2G;
        }
    }
    return -1;
}

cgx_status check_array(const cgx_array& a, int dofs, const char* what) {
    if (!a.data) return fail(CGX_ERR_INVALID_ARG, std::string(what) + ".data is NULL");
    if (!valid_dtype(a.dtype)) return fail(CGX_ERR_INVALID_ARG, std::string(what) + ".dtype must be CGX_F32 or CGX_F64");
    if (a.dofs < dofs) return fail(CGX_ERR_INVALID_ARG, std::string(what) + " has fewer dofs than the operator uses");
    return CGX_OK;
}

// cgx_p2g_adjoint (p2g = true) and cgx_g2p_adjoint (p2g = false).
cgx_status adjoint(cgx_handle h, const cgx_mesh* mesh, const cgx_field* points, int64_t num_point, int spline_order,
                   const cgx_adjoint_op* ops, int n_ops, int precision, const cgx_tiling* tiling,
                   const cgx_field* points_bar, unsigned flags, void* stream, bool p2g) {
    if (!h) return fail(CGX_ERR_INVALID_ARG, "handle is NULL");
    cgx_status s = check_mesh(mesh);
    if (s) return s;
    if (mesh_dims(*mesh) != 3) return fail(CGX_ERR_NOT_SUPPORTED, "adjoints are built for 3D meshes");
    if (num_point < 0) return fail(CGX_ERR_INVALID_ARG, "num_point must be >= 0");
    if (num_point > 0) {
        s = check_field(points, "points");
        if (s) return s;
        if (points->dtype != CGX_F64) return fail(CGX_ERR_INVALID_ARG, "point coordinates must be double (CGX_F64)");
    }
    if (spline_order < 0 || spline_order > 6) return fail(CGX_ERR_NOT_SUPPORTED, "spline order must be in [0, 6]");
    if (precision != CGX_PLAIN_FP64 && precision != CGX_FP32_COMPENSATED)
        return fail(CGX_ERR_INVALID_ARG, "unknown precision");
    if (!ops || n_ops < 1 || n_ops > kMaxOps) return fail(CGX_ERR_INVALID_ARG, "n_ops must be in [1, 8]");
    const bool want_pos = points_bar != nullptr;
    if (want_pos && num_point > 0) {
        s = check_field(points_bar, "points_bar");
        if (s) return s;
    }
    // Validate every operator for the roles it plays in this call.
    for (int o = 0; o < n_ops; ++o) {
        const cgx_adjoint_op& op = ops[o];
        if (adjoint_pattern(op.kind, p2g) < 0) return fail(CGX_ERR_INVALID_ARG, "unknown operator kind");
        const int dofs = p2g ? p2g_dofs(op.kind) : g2p_dofs(op.kind);
        if (p2g) {
            s = check_array(op.array_bar, dofs, "op.array_bar");
            if (s) return s;
            if (num_point > 0 && op.x_bar.data) {
                s = check_field(&op.x_bar, "op.x_bar");
                if (s) return s;
            }
            if (num_point > 0 && want_pos) {
                s = check_field(&op.x, "op.x");
                if (s) return s;
            }
        } else {
            if (num_point > 0) {
                s = check_field(&op.x_bar, "op.x_bar");
                if (s) return s;
            }
            if (op.array_bar.data) {
                s = check_array(op.array_bar, dofs, "op.array_bar");
                if (s) return s;
            }
            if (want_pos) {
                s = check_array(op.array, dofs, "op.array");
                if (s) return s;
            }
        }
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (flags & CGX_FLAG_CHECK_BOUNDS) CGX_CUDA(cudaMemsetAsync(h->flags, 0, sizeof(int), st));
    const unsigned inner = (flags & ~CGX_FLAG_CHECK_BOUNDS) | CGX_FLAG_SKIP_HALO;
    const bool halo = any_periodic(*mesh) && !(flags & CGX_FLAG_SKIP_HALO);

    // The value part is the transposed operator through the forward kernels.
    cgx_op vops[kMaxOps];
    int nv = 0;
    for (int o = 0; o < n_ops; ++o) {
        const cgx_adjoint_op& op = ops[o];
        if (p2g ? !op.x_bar.data : !op.array_bar.data) continue;
        cgx_op& v = vops[nv++];
        std::memset(&v, 0, sizeof(v));
        v.kind = transpose_kind(op.kind, p2g);
        v.multiplier = op.multiplier;
        v.x = op.x_bar;
        v.array = op.array_bar;
    }

    if (p2g && halo) {
        // adjoint of the forward halo scatter(Sum), on each distinct array_bar
        for (int o = 0; o < n_ops; ++o) {
            bool seen = false;
            for (int q = 0; q < o; ++q) seen |= ops[q].array_bar.data == ops[o].array_bar.data;
            if (!seen) CGX_CUDA(launch_halo(to_halo(*mesh, ops[o].array_bar), kHaloGatherAdd, h->sms, st));
        }
    }
    // Value terms (ScalarValue / VectorValue pairings) in the FP32 form with
    // a tiling: dL/dx is the point field against the gradient sums of the
    // array, which the tiled G2P forms (ScalarGradientG2P / VectorGradientG2P
    // into a scratch field), then one combine kernel; other terms take the
    // point kernel.
    bool value_only = want_pos && num_point > 0 && precision == CGX_FP32_COMPENSATED && tiling &&
                      spline_order >= 1 && spline_order <= 3;
    for (int o = 0; o < n_ops && value_only; ++o) {
        const int pat = adjoint_pattern(ops[o].kind, p2g);
        value_only = pat == kAdjValue1 || pat == kAdjValue3;
    }
    if (value_only) {
        const size_t need = size_t(num_point) * 9 * sizeof(float);
        if (need > h->adj_bytes) {
            if (h->adj) cudaFree(h->adj);
            h->adj = nullptr;
            h->adj_bytes = 0;
            if (cudaMalloc(&h->adj, need) != cudaSuccess) return fail(CGX_ERR_NO_MEMORY, "adjoint scratch allocation failed");
            h->adj_bytes = need;
        }
        float* grads = reinterpret_cast<float*>(h->adj);
        for (int o = 0; o < n_ops; ++o) {
            const bool vec = adjoint_pattern(ops[o].kind, p2g) == kAdjValue3;
            const int nc = vec ? 3 : 1;
            CGX_CUDA(cudaMemsetAsync(grads, 0, size_t(num_point) * 3 * nc * sizeof(float), st));
            cgx_op g;
            std::memset(&g, 0, sizeof(g));
            g.kind = vec ? CGX_VECTOR_GRADIENT_G2P : CGX_SCALAR_GRADIENT_G2P;
            g.multiplier = 1.0;
            g.x.data = grads;
            g.x.dtype = CGX_F32;
            g.x.vector_length = 1;
            g.x.soa_stride = 3 * nc;
            g.x.comp_stride = 1;
            g.array = p2g ? ops[o].array_bar : ops[o].array;
            s = interpolate(h, mesh, points, num_point, spline_order, &g, 1, precision, tiling, inner, stream, false);
            if (s) return s;
            const cgx_field& sf = p2g ? ops[o].x : ops[o].x_bar;
            CGX_CUDA(launch_adjoint_value_combine(to_dfield(*points_bar), to_dfield(sf), grads, num_point, nc,
                                                  float(ops[o].multiplier), h->sms, st));
        }
    } else if (want_pos && num_point > 0) {
        AdjointParams prm;
        std::memset(&prm, 0, sizeof(prm));
        prm.mesh = to_dmesh(*mesh);
        prm.points = to_dfield(*points);
        prm.points_bar = to_dfield(*points_bar);
        prm.num_point = num_point;
        prm.n_terms = n_ops;
        prm.error_flag = h->flags;
        for (int o = 0; o < n_ops; ++o) {
            AdjointTerm& t = prm.terms[o];
            t.pattern = adjoint_pattern(ops[o].kind, p2g);
            t.mult = ops[o].multiplier;
            t.mult_f = float(ops[o].multiplier);
            const cgx_field& sf = p2g ? ops[o].x : ops[o].x_bar;
            const cgx_array& af = p2g ? ops[o].array_bar : ops[o].array;
            t.s = to_dfield(sf);
            t.a.data = reinterpret_cast<char*>(af.data);
            t.a.dtype = af.dtype;
            t.a.dofs = af.dofs;
        }
        CGX_CUDA(launch_adjoint_points(prm, spline_order, precision == CGX_PLAIN_FP64, h->sms, st));
    }
    if (nv > 0 && num_point > 0) {
        s = interpolate(h, mesh, points, num_point, spline_order, vops, nv, precision, tiling, inner, stream, !p2g);
        if (s) return s;
    }
    if (!p2g && halo) {
        // adjoint of the forward halo gather, on each distinct array_bar
        for (int o = 0; o < nv; ++o) {
            bool seen = false;
            for (int q = 0; q < o; ++q) seen |= vops[q].array.data == vops[o].array.data;
            if (!seen) CGX_CUDA(launch_halo(to_halo(*mesh, vops[o].array), kHaloScatterClear, h->sms, st));
        }
    }
    return finish_check(h, flags, st);
}

int key_bits_for(int64_t nbin) {
    int b = 0;
    while ((int64_t(1) << b) < nbin) ++b;
    return b;
}

char* align256(char* p) { return reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 255) / 256 * 256); }

}  // namespace

extern "C" {

cgx_status cgx_create(cgx_handle* out) {
    if (!out) return fail(CGX_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    cgx_context* h = new cgx_context();
    cudaError_t e = cudaGetDevice(&h->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device);
    if (e == cudaSuccess) e = cudaMalloc(&h->flags, 64);
    if (e == cudaSuccess) e = cudaMemset(h->flags, 0, 64);
    if (e != cudaSuccess) {
        if (h->flags) cudaFree(h->flags);
        delete h;
        return cuda_fail(e, "cgx_create");
    }
    *out = h;
    return CGX_OK;
}

cgx_status cgx_destroy(cgx_handle h) {
    if (!h) return CGX_OK;
    if (h->ws) cudaFree(h->ws);
    if (h->flags) cudaFree(h->flags);
    if (h->work) cudaFree(h->work);
    if (h->work_prefix) cudaFree(h->work_prefix);
    if (h->adj) cudaFree(h->adj);
    delete h;
    return CGX_OK;
}

const char* cgx_last_error(void) { return g_last_error.c_str(); }

const char* cgx_version(void) { return "cgx 0.1 (sm_103a)"; }

}  // extern "C"

void cgx::set_last_error(const char* msg) { g_last_error = msg; }

extern "C" {

int cgx_last_dispatch(cgx_handle h) { return h ? h->last_dispatch : CGX_DISPATCH_NONE; }

cgx_status cgx_p2g(cgx_handle h, const cgx_mesh* mesh, const cgx_field* points, int64_t num_point, int spline_order,
                   const cgx_op* ops, int n_ops, int precision, const cgx_tiling* tiling, unsigned flags,
                   void* stream) {
    return interpolate(h, mesh, points, num_point, spline_order, ops, n_ops, precision, tiling, flags, stream, true);
}

cgx_status cgx_g2p(cgx_handle h, const cgx_mesh* mesh, const cgx_field* points, int64_t num_point, int spline_order,
                   const cgx_op* ops, int n_ops, int precision, const cgx_tiling* tiling, unsigned flags,
                   void* stream) {
    return interpolate(h, mesh, points, num_point, spline_order, ops, n_ops, precision, tiling, flags, stream, false);
}

cgx_status cgx_g2p2g(cgx_handle h, const cgx_mesh* mesh, const cgx_field* points, int64_t num_point, int spline_order,
                     const cgx_op* g2p_ops, int n_g2p, const cgx_op* p2g_ops, int n_p2g, int precision,
                     const cgx_tiling* tiling, unsigned flags, void* stream) {
    if (!h) return fail(CGX_ERR_INVALID_ARG, "handle is NULL");
    cgx_status s = check_mesh(mesh);
    if (s) return s;
    if (mesh_dims(*mesh) != 3) return fail(CGX_ERR_NOT_SUPPORTED, "g2p2g is built for 3D meshes");
    if (num_point < 0) return fail(CGX_ERR_INVALID_ARG, "num_point must be >= 0");
    if (num_point > 0) {
        s = check_field(points, "points");
        if (s) return s;
        if (points->dtype != CGX_F64) return fail(CGX_ERR_INVALID_ARG, "point coordinates must be double (CGX_F64)");
    }
    if (spline_order < 0 || spline_order > 6) return fail(CGX_ERR_NOT_SUPPORTED, "spline order must be in [0, 6]");
    if (precision != CGX_PLAIN_FP64 && precision != CGX_FP32_COMPENSATED)
        return fail(CGX_ERR_INVALID_ARG, "unknown precision");
    if (n_g2p < 1 || n_p2g < 1 || n_g2p + n_p2g > kMaxOps)
        return fail(CGX_ERR_INVALID_ARG, "g2p2g takes >= 1 G2P and >= 1 P2G functor, 8 in all");
    s = check_ops(g2p_ops, n_g2p, false, num_point > 0);
    if (s) return s;
    s = check_ops(p2g_ops, n_p2g, true, num_point > 0);
    if (s) return s;
    if (tiling && precision == CGX_FP32_COMPENSATED && num_point > 0) {
        // G2P completes over all points before P2G writes: the same contract
        // as the fused kernel, with the tiled kernels where they apply
        s = interpolate(h, mesh, points, num_point, spline_order, g2p_ops, n_g2p, precision, tiling, flags, stream,
                        false);
        if (s) return s;
        const int g2p_dispatch = h->last_dispatch;
        s = interpolate(h, mesh, points, num_point, spline_order, p2g_ops, n_p2g, precision, tiling, flags, stream,
                        true);
        if (!s && g2p_dispatch != CGX_DISPATCH_TILED) h->last_dispatch = g2p_dispatch;
        return s;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (flags & CGX_FLAG_CHECK_BOUNDS) CGX_CUDA(cudaMemsetAsync(h->flags, 0, sizeof(int), st));
    if (!(flags & CGX_FLAG_SKIP_HALO)) {
        s = halo_all(*mesh, g2p_ops, n_g2p, kHaloGather, h->sms, st);
        if (s) return s;
    }
    const DMesh dm = to_dmesh(*mesh);
    const int64_t nodes = int64_t(dm.ext[0]) * dm.ext[1] * dm.ext[2];
    // G2P reads each array as it was at the call: an array that a P2G functor
    // also writes is read from a snapshot in the workspace.
    std::vector<cgx_op> gops(g2p_ops, g2p_ops + n_g2p);
    std::vector<size_t> snap_off(n_g2p, size_t(-1));
    size_t snap_bytes = 0;
    for (int o = 0; o < n_g2p; ++o) {
        bool written = false;
        for (int q = 0; q < n_p2g; ++q) written |= p2g_ops[q].array.data == gops[o].array.data;
        if (!written) continue;
        for (int q = 0; q < o; ++q)
            if (g2p_ops[q].array.data == gops[o].array.data) snap_off[o] = snap_off[q];
        if (snap_off[o] != size_t(-1)) continue;
        snap_off[o] = snap_bytes;
        const size_t bytes = size_t(nodes) * gops[o].array.dofs * (gops[o].array.dtype == CGX_F64 ? 8 : 4);
        snap_bytes += (bytes + 255) / 256 * 256;
    }
    if (snap_bytes > 0 && num_point > 0) {
        s = ensure_ws(h, snap_bytes);
        if (s) return s;
        for (int o = 0; o < n_g2p; ++o) {
            if (snap_off[o] == size_t(-1)) continue;
            char* snap = reinterpret_cast<char*>(h->ws) + snap_off[o];
            bool first = true;
            for (int q = 0; q < o; ++q) first &= snap_off[q] != snap_off[o];
            if (first) {
                const size_t bytes = size_t(nodes) * gops[o].array.dofs * (gops[o].array.dtype == CGX_F64 ? 8 : 4);
                CGX_CUDA(cudaMemcpyAsync(snap, gops[o].array.data, bytes, cudaMemcpyDeviceToDevice, st));
            }
            gops[o].array.data = snap;
        }
    }
    if (num_point > 0) {
        PointParams prm;
        std::memset(&prm, 0, sizeof(prm));
        prm.mesh = dm;
        prm.points = to_dfield(*points);
        prm.num_point = num_point;
        prm.n_ops = n_g2p + n_p2g;
        prm.n_g2p = n_g2p;
        prm.dims = 3;
        prm.error_flag = h->flags;
        for (int o = 0; o < prm.n_ops; ++o) {
            const cgx_op& op = o < n_g2p ? gops[o] : p2g_ops[o - n_g2p];
            prm.ops[o].kind = op.kind;
            prm.ops[o].slot = o;
            prm.ops[o].mult = op.multiplier;
            prm.ops[o].mult_f = float(op.multiplier);
            prm.ops[o].x = to_dfield(op.x);
            prm.ops[o].a.data = reinterpret_cast<char*>(op.array.data);
            prm.ops[o].a.dtype = op.array.dtype;
            prm.ops[o].a.dofs = op.array.dofs;
        }
        CGX_CUDA(launch_g2p2g_points(prm, spline_order, precision == CGX_PLAIN_FP64, h->sms, st));
        h->last_dispatch = CGX_DISPATCH_POINTS;
    }
    if (!(flags & CGX_FLAG_SKIP_HALO)) {
        s = halo_all(*mesh, p2g_ops, n_p2g, kHaloScatterSum, h->sms, st);
        if (s) return s;
    }
    return finish_check(h, flags, st);
}

cgx_status cgx_p2g_adjoint(cgx_handle h, const cgx_mesh* mesh, const cgx_field* points, int64_t num_point,
                           int spline_order, const cgx_adjoint_op* ops, int n_ops, int precision,
                           const cgx_tiling* tiling, const cgx_field* points_bar, unsigned flags, void* stream) {
    return adjoint(h, mesh, points, num_point, spline_order, ops, n_ops, precision, tiling, points_bar, flags, stream,
                   true);
}

cgx_status cgx_g2p_adjoint(cgx_handle h, const cgx_mesh* mesh, const cgx_field* points, int64_t num_point,
                           int spline_order, const cgx_adjoint_op* ops, int n_ops, int precision,
                           const cgx_tiling* tiling, const cgx_field* points_bar, unsigned flags, void* stream) {
    return adjoint(h, mesh, points, num_point, spline_order, ops, n_ops, precision, tiling, points_bar, flags, stream,
                   false);
}

cgx_status cgx_halo_scatter_sum(const cgx_mesh* mesh, const cgx_array* array, void* stream) {
    cgx_status s = check_mesh(mesh);
    if (s) return s;
    if (!array || !array->data || !valid_dtype(array->dtype) || array->dofs < 1)
        return fail(CGX_ERR_INVALID_ARG, "bad array");
    if (!any_periodic(*mesh)) return CGX_OK;
    int dev = 0, sms = 0;
    CGX_CUDA(cudaGetDevice(&dev));
    CGX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CGX_CUDA(launch_halo(to_halo(*mesh, *array), kHaloScatterSum, sms, reinterpret_cast<cudaStream_t>(stream)));
    return CGX_OK;
}

cgx_status cgx_halo_gather(const cgx_mesh* mesh, const cgx_array* array, void* stream) {
    cgx_status s = check_mesh(mesh);
    if (s) return s;
    if (!array || !array->data || !valid_dtype(array->dtype) || array->dofs < 1)
        return fail(CGX_ERR_INVALID_ARG, "bad array");
    if (!any_periodic(*mesh)) return CGX_OK;
    int dev = 0, sms = 0;
    CGX_CUDA(cudaGetDevice(&dev));
    CGX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CGX_CUDA(launch_halo(to_halo(*mesh, *array), kHaloGather, sms, reinterpret_cast<cudaStream_t>(stream)));
    return CGX_OK;
}

cgx_status cgx_array_assign(const cgx_mesh* mesh, const cgx_array* array, double value, void* stream) {
    cgx_status s = check_mesh(mesh);
    if (s) return s;
    if (!array || !array->data || !valid_dtype(array->dtype) || array->dofs < 1)
        return fail(CGX_ERR_INVALID_ARG, "bad array");
    const DMesh dm = to_dmesh(*mesh);
    const int64_t count = int64_t(dm.ext[0]) * dm.ext[1] * dm.ext[2] * array->dofs;
    int dev = 0, sms = 0;
    CGX_CUDA(cudaGetDevice(&dev));
    CGX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CGX_CUDA(launch_fill(array->data, array->dtype, count, value, sms, reinterpret_cast<cudaStream_t>(stream)));
    return CGX_OK;
}

cgx_status cgx_cartesian_num_bins(const double grid_min[3], const double grid_max[3], const double grid_delta[3],
                                  int32_t nbin_out[3]) {
    if (!grid_min || !grid_max || !grid_delta || !nbin_out) return fail(CGX_ERR_INVALID_ARG, "NULL argument");
    for (int d = 0; d < 3; ++d) {
        if (!(grid_delta[d] > 0.0) || !(grid_max[d] > grid_min[d]))
            return fail(CGX_ERR_INVALID_ARG, "grid bounds / delta invalid");
        // cellsBetween(max, min, 1 / delta) = floor((max - min) * (1 / delta))
        nbin_out[d] = int32_t(std::floor((grid_max[d] - grid_min[d]) * (1.0 / grid_delta[d])));
        if (nbin_out[d] < 1) return fail(CGX_ERR_INVALID_ARG, "grid has no cells");
    }
    return CGX_OK;
}

}  // extern "C"

namespace {

// LinkedCellList::build for `dims` (2 or 3) coordinates; grid arrays have
// `dims` entries.
cgx_status linked_cell_build(cgx_handle h, const cgx_field* positions, int dims, int64_t begin, int64_t end,
                             const double* grid_min, const double* grid_max, const double* grid_delta,
                             int32_t* counts, uint64_t* offsets, uint64_t* permutes, void* stream) {
    if (!h) return fail(CGX_ERR_INVALID_ARG, "handle is NULL");
    cgx_status s = check_field(positions, "positions");
    if (s) return s;
    if (positions->dtype != CGX_F64) return fail(CGX_ERR_INVALID_ARG, "positions must be double");
    if (begin < 0 || end < begin) return fail(CGX_ERR_INVALID_ARG, "need 0 <= begin <= end");
    if (end - begin >= (int64_t(1) << 32)) return fail(CGX_ERR_NOT_SUPPORTED, "more than 2^32 - 1 particles");
    if (!counts || !offsets || (!permutes && end > begin)) return fail(CGX_ERR_INVALID_ARG, "NULL output");
    if (!grid_min || !grid_max || !grid_delta) return fail(CGX_ERR_INVALID_ARG, "NULL argument");
    // Pad a 2D grid with one z cell of width 1 (never read by the key kernel).
    double gmin[3] = {0.0, 0.0, 0.0}, gmax[3] = {1.0, 1.0, 1.0}, gdel[3] = {1.0, 1.0, 1.0};
    for (int d = 0; d < dims; ++d) {
        gmin[d] = grid_min[d];
        gmax[d] = grid_max[d];
        gdel[d] = grid_delta[d];
    }
    int32_t nx[3];
    s = cgx_cartesian_num_bins(gmin, gmax, gdel, nx);
    if (s) return s;
    const int64_t ncell = int64_t(nx[0]) * nx[1] * nx[2];
    if (ncell >= (int64_t(1) << 31)) return fail(CGX_ERR_NOT_SUPPORTED, "more than 2^31 bins");
    double mn[3], rdx[3];
    for (int d = 0; d < 3; ++d) {
        mn[d] = gmin[d];
        const double dx = (gmax[d] - gmin[d]) / nx[d];
        rdx[d] = 1.0 / dx;
    }
    const int64_t n = end - begin;
    const size_t need = size_t(n) * 4 + 256 + radix_sort_scratch_bytes(n) + scan_scratch_bytes(ncell) + 1024;
    s = ensure_ws(h, need);
    if (s) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    char* p = reinterpret_cast<char*>(h->ws);
    uint32_t* keys = reinterpret_cast<uint32_t*>(p);
    p = align256(p + size_t(n) * 4);
    void* scratch = p;
    CGX_CUDA(cudaMemsetAsync(h->flags, 0, sizeof(int), st));
    CGX_CUDA(cudaMemsetAsync(counts, 0, size_t(ncell) * sizeof(int32_t), st));
    CGX_CUDA(cartesian_keys(to_dfield(*positions), dims, begin, end, mn, rdx, nx, keys, counts, h->flags, st,
                            h->sms));
    CGX_CUDA(exclusive_scan_counts(counts, ncell, offsets, nullptr, scratch, h->sms, st));
    if (n > 0)
        CGX_CUDA(radix_sort_pairs(keys, n, key_bits_for(ncell), permutes, nullptr, uint64_t(begin), scratch,
                                  radix_sort_scratch_bytes(n), h->sms, st));
    return CGX_OK;
}

}  // namespace

extern "C" {

cgx_status cgx_linked_cell_build(cgx_handle h, const cgx_field* positions, int64_t begin, int64_t end,
                                 const double grid_min[3], const double grid_max[3], const double grid_delta[3],
                                 int32_t* counts, uint64_t* offsets, uint64_t* permutes, void* stream) {
    return linked_cell_build(h, positions, 3, begin, end, grid_min, grid_max, grid_delta, counts, offsets, permutes,
                             stream);
}

cgx_status cgx_linked_cell_build_2d(cgx_handle h, const cgx_field* positions, int64_t begin, int64_t end,
                                    const double grid_min[2], const double grid_max[2], const double grid_delta[2],
                                    int32_t* counts, uint64_t* offsets, uint64_t* permutes, void* stream) {
    return linked_cell_build(h, positions, 2, begin, end, grid_min, grid_max, grid_delta, counts, offsets, permutes,
                             stream);
}

cgx_status cgx_bin_by_key(cgx_handle h, const int32_t* keys, int64_t begin, int64_t end, int32_t nbin,
                          int32_t* counts, uint64_t* offsets, uint64_t* permutes, void* stream) {
    if (!h) return fail(CGX_ERR_INVALID_ARG, "handle is NULL");
    if (begin < 0 || end < begin) return fail(CGX_ERR_INVALID_ARG, "need 0 <= begin <= end");
    if (nbin < 1) return fail(CGX_ERR_INVALID_ARG, "nbin must be >= 1");
    if ((!keys || !permutes) && end > begin) return fail(CGX_ERR_INVALID_ARG, "NULL keys / permutes");
    if (!counts || !offsets) return fail(CGX_ERR_INVALID_ARG, "NULL output");
    if (end - begin >= (int64_t(1) << 32)) return fail(CGX_ERR_NOT_SUPPORTED, "more than 2^32 - 1 keys");
    const int64_t n = end - begin;
    const size_t need = size_t(n) * 4 + 256 + radix_sort_scratch_bytes(n) + scan_scratch_bytes(nbin) + 1024;
    cgx_status s = ensure_ws(h, need);
    if (s) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    char* p = reinterpret_cast<char*>(h->ws);
    uint32_t* k32 = reinterpret_cast<uint32_t*>(p);
    p = align256(p + size_t(n) * 4);
    void* scratch = p;
    CGX_CUDA(cudaMemsetAsync(h->flags, 0, sizeof(int), st));
    CGX_CUDA(cudaMemsetAsync(counts, 0, size_t(nbin) * sizeof(int32_t), st));
    CGX_CUDA(key_histogram(keys, begin, end, k32, counts, nbin, h->flags, st, h->sms));
    CGX_CUDA(exclusive_scan_counts(counts, nbin, offsets, nullptr, scratch, h->sms, st));
    if (n > 0)
        CGX_CUDA(radix_sort_pairs(k32, n, key_bits_for(nbin), permutes, nullptr, uint64_t(begin), scratch,
                                  radix_sort_scratch_bytes(n), h->sms, st));
    return finish_check(h, CGX_FLAG_CHECK_BOUNDS, st);
}

cgx_status cgx_bin_by_key_range(cgx_handle h, const int32_t* keys, int64_t begin, int64_t end, int32_t nbin,
                                int sort_within_bins, int32_t* counts, uint64_t* offsets, uint64_t* permutes,
                                void* stream) {
    if (!h) return fail(CGX_ERR_INVALID_ARG, "handle is NULL");
    if (begin < 0 || end < begin) return fail(CGX_ERR_INVALID_ARG, "need 0 <= begin <= end");
    if (nbin < 0 || nbin == INT32_MAX) return fail(CGX_ERR_INVALID_ARG, "need 0 <= nbin < 2^31 - 1");
    if ((!keys || !permutes) && end > begin) return fail(CGX_ERR_INVALID_ARG, "NULL keys / permutes");
    if (!counts || !offsets) return fail(CGX_ERR_INVALID_ARG, "NULL output");
    if (end - begin >= (int64_t(1) << 32)) return fail(CGX_ERR_NOT_SUPPORTED, "more than 2^32 - 1 keys");
    const int64_t n = end - begin;
    const int32_t nbins = nbin + 1;  // Kokkos::BinOp1D::max_bins
    const size_t need = size_t(n) * 4 + 256 + 256 + radix_sort_scratch_bytes(n) + scan_scratch_bytes(nbins) + 1024;
    cgx_status s = ensure_ws(h, need);
    if (s) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    char* p = reinterpret_cast<char*>(h->ws);
    uint32_t* k32 = reinterpret_cast<uint32_t*>(p);
    p = align256(p + size_t(n) * 4);
    int* minmax = reinterpret_cast<int*>(p);
    p = align256(p + 2 * sizeof(int));
    void* scratch = p;
    CGX_CUDA(cudaMemsetAsync(counts, 0, size_t(nbins) * sizeof(int32_t), st));
    if (n == 0) {
        CGX_CUDA(exclusive_scan_counts(counts, nbins, offsets, nullptr, scratch, h->sms, st));
        return CGX_OK;
    }
    // The key range sets the bin width, so it is read back first (the
    // reference's keyMinMax is a blocking reduction too).
    CGX_CUDA(key_minmax(keys, begin, end, minmax, st, h->sms));
    int mm[2] = {0, 0};
    CGX_CUDA(cudaMemcpyAsync(mm, minmax, sizeof(mm), cudaMemcpyDeviceToHost, st));
    CGX_CUDA(cudaStreamSynchronize(st));
    // Kokkos::BinOp1D(nbin, min, max) for integer keys: nbin / (max - min)
    // keys per bin, or one key value per bin when the range is at most nbin.
    const double range = double(mm[1]) - double(mm[0]);
    const double mul = range <= double(nbin) ? 1.0 : double(nbin) / range;
    const bool by_key = sort_within_bins != 0;
    CGX_CUDA(key_bin1d(keys, begin, end, mm[0], mul, nbins, by_key, k32, counts, st, h->sms));
    CGX_CUDA(exclusive_scan_counts(counts, nbins, offsets, nullptr, scratch, h->sms, st));
    const int bits = by_key ? key_bits_for(int64_t(mm[1]) - int64_t(mm[0]) + 1) : key_bits_for(nbins);
    CGX_CUDA(radix_sort_pairs(k32, n, bits, permutes, nullptr, uint64_t(begin), scratch, radix_sort_scratch_bytes(n),
                              h->sms, st));
    return CGX_OK;
}

cgx_status cgx_permute(cgx_handle h, const uint64_t* permutes, int64_t begin, int64_t end, const cgx_field* fields,
                       const int32_t* ncomps, int n_fields, void* stream) {
    if (!h) return fail(CGX_ERR_INVALID_ARG, "handle is NULL");
    if (begin < 0 || end < begin) return fail(CGX_ERR_INVALID_ARG, "need 0 <= begin <= end");
    if (end == begin) return CGX_OK;
    if (!permutes || !fields || !ncomps || n_fields < 1) return fail(CGX_ERR_INVALID_ARG, "NULL argument");
    size_t need = 0;
    for (int f = 0; f < n_fields; ++f) {
        cgx_status s = check_field(&fields[f], "field");
        if (s) return s;
        if (ncomps[f] < 1) return fail(CGX_ERR_INVALID_ARG, "ncomps must be >= 1");
        const size_t b = size_t(end - begin) * ncomps[f] * (fields[f].dtype == CGX_F64 ? 8 : 4);
        if (b > need) need = b;
    }
    cgx_status s = ensure_ws(h, need);
    if (s) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    for (int f = 0; f < n_fields; ++f)
        CGX_CUDA(permute_field(permutes, begin, end, to_dfield(fields[f]), ncomps[f], h->ws, st, h->sms));
    return CGX_OK;
}

cgx_status cgx_tiling_init(const cgx_mesh* mesh, int spline_order, const int32_t tile[3], cgx_tiling* out) {
    cgx_status s = check_mesh(mesh);
    if (s) return s;
    if (mesh_dims(*mesh) != 3) return fail(CGX_ERR_NOT_SUPPORTED, "tilings are built for 3D meshes");
    if (!tile || !out) return fail(CGX_ERR_INVALID_ARG, "NULL argument");
    if (spline_order < 0 || spline_order > 6) return fail(CGX_ERR_NOT_SUPPORTED, "spline order must be in [0, 6]");
    const DMesh dm = to_dmesh(*mesh);
    int64_t total = 1;
    for (int d = 0; d < 3; ++d) {
        if (tile[d] < 1 || tile[d] > 64) return fail(CGX_ERR_INVALID_ARG, "tile extent must be in [1, 64]");
        out->tile[d] = tile[d];
        // base nodes range over [0, ext - num_knot]
        const int nbase = dm.ext[d] - spline_order;
        out->num_tiles[d] = nbase < 1 ? 1 : (nbase + tile[d] - 1) / tile[d];
        total *= out->num_tiles[d];
    }
    if (total * tile[0] * tile[1] * tile[2] >= (int64_t(1) << 32))
        return fail(CGX_ERR_NOT_SUPPORTED, "tiling has more than 2^32 base nodes");
    out->spline_order = spline_order;
    out->reserved = 0;
    out->tile_offsets = nullptr;
    return CGX_OK;
}

int64_t cgx_tiling_num_offsets(const cgx_tiling* t) {
    if (!t) return 0;
    return int64_t(t->num_tiles[0]) * t->num_tiles[1] * t->num_tiles[2] + 1;
}

cgx_status cgx_sort_tiles(cgx_handle h, const cgx_mesh* mesh, const cgx_field* points, int64_t num_point,
                          cgx_tiling* tiling, uint64_t* permutes, void* stream) {
    if (!h) return fail(CGX_ERR_INVALID_ARG, "handle is NULL");
    cgx_status s = check_mesh(mesh);
    if (s) return s;
    if (mesh_dims(*mesh) != 3) return fail(CGX_ERR_NOT_SUPPORTED, "tilings are built for 3D meshes");
    s = check_field(points, "points");
    if (s) return s;
    if (points->dtype != CGX_F64) return fail(CGX_ERR_INVALID_ARG, "point coordinates must be double");
    if (!tiling || !tiling->tile_offsets) return fail(CGX_ERR_INVALID_ARG, "tiling / tile_offsets is NULL");
    if (num_point < 0 || num_point >= (int64_t(1) << 32)) return fail(CGX_ERR_NOT_SUPPORTED, "num_point out of range");
    if (num_point > 0 && !permutes) return fail(CGX_ERR_INVALID_ARG, "permutes is NULL");
    const int64_t nt = cgx_tiling_num_offsets(tiling) - 1;
    const int64_t cpt = int64_t(tiling->tile[0]) * tiling->tile[1] * tiling->tile[2];
    const size_t need = size_t(num_point) * 4 + 256 + size_t(nt) * 4 + 256 + radix_sort_scratch_bytes(num_point) +
                        size_t(nt) * 8 + scan_scratch_bytes(nt) + 4096;
    s = ensure_ws(h, need);
    if (s) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    char* p = reinterpret_cast<char*>(h->ws);
    uint32_t* keys = reinterpret_cast<uint32_t*>(p);
    p = align256(p + size_t(num_point) * 4);
    int32_t* tcounts = reinterpret_cast<int32_t*>(p);
    p = align256(p + size_t(nt) * 4);
    void* scratch = p;
    const DMesh dm = to_dmesh(*mesh);
    CGX_CUDA(cudaMemsetAsync(tcounts, 0, size_t(nt) * 4, st));
    CGX_CUDA(tile_keys(dm, to_dfield(*points), num_point, tiling->spline_order, tiling->tile, tiling->num_tiles, keys,
                       tcounts, st, h->sms));
    CGX_CUDA(counts_to_int64_offsets(tcounts, nt, tiling->tile_offsets, scratch, st, h->sms));
    if (num_point > 0)
        CGX_CUDA(radix_sort_pairs(keys, num_point, key_bits_for(nt * cpt), permutes, nullptr, 0, scratch,
                                  radix_sort_scratch_bytes(num_point), h->sms, st));
    return CGX_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched launches: many independent meshes, one work list, one persistent
// kernel per direction (per distinct array for g2p).
// ---------------------------------------------------------------------------
struct cgx_batch {
    cgx_context* h = nullptr;
    bool p2g = true;
    int order = 2;
    int n_inst = 0;
    TiledParams prm;                   // operator structure; instances -> geoms
    std::vector<cgx_mesh> meshes;      // for the halo step
    std::vector<cgx_array> arrays;     // n_inst x n_arrays distinct arrays
    bool any_periodic = false;
    int64_t total_tiles = 0;
    int64_t total_points = 0;
    TiledGeom* geoms = nullptr;        // device
    const int64_t** offs = nullptr;    // device: per-instance tile offsets
    int64_t* tile_base = nullptr;      // device: n_inst + 1
    WorkItem* work = nullptr;
    size_t work_cap = 0;
    int64_t* work_prefix = nullptr;
    void* scratch = nullptr;
    int* flags = nullptr;              // [0] error, [1] counter, [2..3] work count
    size_t box_bytes = 0;              // p2g node boxes
    std::vector<size_t> slot_smem;     // g2p dynamic shared memory per slot
    int max_per_sm = 1;                // resident CTAs per SM (all launches of the plan)
    int ctas_per_sm = 1;
    int64_t item = 0;                  // particles per work item
};

namespace {

constexpr int64_t kMinBatchItem = 256;

void batch_free(cgx_batch* b) {
    if (!b) return;
    cudaFree(b->geoms);
    cudaFree(b->offs);
    cudaFree(b->tile_base);
    cudaFree(b->work);
    cudaFree(b->work_prefix);
    cudaFree(b->scratch);
    cudaFree(b->flags);
    delete b;
}

cgx_status batch_run(cgx_batch* b, unsigned flags, cudaStream_t st) {
    const TiledParams& prm = b->prm;
    const bool halo = b->any_periodic && !(flags & CGX_FLAG_SKIP_HALO);
    const int n_arrays = prm.n_arrays;
    if (flags & CGX_FLAG_CHECK_BOUNDS) CGX_CUDA(cudaMemsetAsync(b->flags, 0, sizeof(int), st));
    if (!b->p2g && halo)
        for (int i = 0; i < b->n_inst; ++i)
            if (::any_periodic(b->meshes[i]))
                for (int a = 0; a < n_arrays; ++a)
                    CGX_CUDA(launch_halo(to_halo(b->meshes[i], b->arrays[size_t(i) * n_arrays + a]), kHaloGather,
                                         b->h->sms, st));
    CGX_CUDA(build_batch_work_items(b->offs, b->tile_base, b->n_inst, b->total_tiles, b->item, b->work_prefix, b->work,
                                    reinterpret_cast<int64_t*>(b->flags + 2), b->scratch, st, b->h->sms));
    const int blocks = b->h->sms * b->ctas_per_sm;
    if (b->p2g) {
        CGX_CUDA(cudaMemsetAsync(b->flags + 1, 0, sizeof(int), st));
        CGX_CUDA(launch_p2g_tiled_prepared(prm, b->order, true, blocks, b->box_bytes, st));
    } else {
        for (int a = 0; a < n_arrays; ++a) {
            TiledParams one = prm;
            one.arrays[a].smem_offset = 0;
            CGX_CUDA(cudaMemsetAsync(b->flags + 1, 0, sizeof(int), st));
            CGX_CUDA(launch_g2p_tiled_prepared(one, b->order, a, true, blocks, b->slot_smem[a], st));
        }
    }
    if (b->p2g && halo)
        for (int i = 0; i < b->n_inst; ++i)
            if (::any_periodic(b->meshes[i]))
                for (int a = 0; a < n_arrays; ++a)
                    CGX_CUDA(launch_halo(to_halo(b->meshes[i], b->arrays[size_t(i) * n_arrays + a]),
                                         kHaloScatterSum, b->h->sms, st));
    if (flags & CGX_FLAG_CHECK_BOUNDS) {
        int host_flag = 0;
        CGX_CUDA(cudaMemcpyAsync(&host_flag, b->flags, sizeof(int), cudaMemcpyDeviceToHost, st));
        CGX_CUDA(cudaStreamSynchronize(st));
        if (host_flag & (1 << CGX_ERR_OUT_OF_BOUNDS))
            return fail(CGX_ERR_OUT_OF_BOUNDS, "a point's stencil left the ghosted index space; it was skipped");
    }
    return CGX_OK;
}

}  // namespace

extern "C" {

cgx_status cgx_batch_plan_create(cgx_handle h, const cgx_instance* inst, int n_inst, int spline_order,
                                 const cgx_op* ops, int n_ops, int p2g, cgx_batch_plan* out) {
    if (!out) return fail(CGX_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!h) return fail(CGX_ERR_INVALID_ARG, "handle is NULL");
    if (!inst || n_inst < 1) return fail(CGX_ERR_INVALID_ARG, "need at least one instance");
    if (spline_order < 1 || spline_order > 3) return fail(CGX_ERR_NOT_SUPPORTED, "batched launches take spline order 1-3");
    if (!ops || n_ops < 1 || n_ops > CGX_BATCH_MAX_OPS) return fail(CGX_ERR_INVALID_ARG, "n_ops must be in [1, 8]");
    const bool is_p2g = p2g != 0;
    // Per instance: the cgx_op list with its own buffers; checks as cgx_p2g / cgx_g2p.
    std::vector<cgx_op> iops(size_t(n_inst) * n_ops);
    for (int i = 0; i < n_inst; ++i) {
        const cgx_instance& I = inst[i];
        cgx_status s = check_mesh(&I.mesh);
        if (!s && mesh_dims(I.mesh) != 3) s = fail(CGX_ERR_NOT_SUPPORTED, "batched launches are built for 3D meshes");
        if (s) return s;
        if (I.num_point < 0) return fail(CGX_ERR_INVALID_ARG, "num_point must be >= 0");
        s = check_field(&I.points, "points");
        if (s) return s;
        if (I.points.dtype != CGX_F64) return fail(CGX_ERR_INVALID_ARG, "point coordinates must be double (CGX_F64)");
        if (!I.tiling.tile_offsets || I.tiling.spline_order != spline_order || I.tiling.tile[0] != kTiledTile ||
            I.tiling.tile[1] != kTiledTile || I.tiling.tile[2] != kTiledTile)
            return fail(CGX_ERR_INVALID_ARG, "every instance needs a tiling of this spline order with tile 8x8x8");
        for (int o = 0; o < n_ops; ++o) {
            cgx_op& op = iops[size_t(i) * n_ops + o];
            op = ops[o];
            op.x = I.x[o];
            op.array = I.array[o];
        }
        s = check_ops(&iops[size_t(i) * n_ops], n_ops, is_p2g, true);
        if (s) return s;
    }
    cgx_batch* b = new cgx_batch();
    b->h = h;
    b->p2g = is_p2g;
    b->order = spline_order;
    b->n_inst = n_inst;
    if (!setup_tiled(b->prm, iops.data(), n_ops, spline_order, is_p2g)) {
        delete b;
        return fail(CGX_ERR_NOT_SUPPORTED, "the operators do not fit the tiled kernels (FP32 point fields, shared memory)");
    }
    const int n_arrays = b->prm.n_arrays;
    std::vector<TiledGeom> geoms(n_inst);
    std::vector<const int64_t*> offs(n_inst);
    std::vector<int64_t> base(size_t(n_inst) + 1, 0);
    b->meshes.resize(n_inst);
    b->arrays.resize(size_t(n_inst) * n_arrays);
    for (int i = 0; i < n_inst; ++i) {
        const cgx_op* io = &iops[size_t(i) * n_ops];
        TiledParams mine;
        setup_tiled(mine, io, n_ops, spline_order, is_p2g);
        for (int o = 0; o < n_ops; ++o) {
            const int slot = b->prm.ops[o].slot;
            if (mine.ops[o].slot != slot || io[o].array.dofs != iops[o].array.dofs ||
                io[o].array.dtype != iops[o].array.dtype || io[o].x.dtype != iops[o].x.dtype) {
                delete b;
                return fail(CGX_ERR_INVALID_ARG, "instances differ in array sharing, dofs or dtypes");
            }
            b->arrays[size_t(i) * n_arrays + slot] = io[o].array;
        }
        if (!fill_geom(geoms[i], b->prm, inst[i].mesh, inst[i].points, io, n_ops, inst[i].tiling, spline_order)) {
            delete b;
            return fail(CGX_ERR_NOT_SUPPORTED, "an instance's mesh origin or extent is beyond the tiled kernels' range");
        }
        b->meshes[i] = inst[i].mesh;
        b->any_periodic |= ::any_periodic(inst[i].mesh);
        offs[i] = inst[i].tiling.tile_offsets;
        const int64_t nt = cgx_tiling_num_offsets(&inst[i].tiling) - 1;
        base[i + 1] = base[i] + nt;
        b->total_points += inst[i].num_point;
    }
    b->total_tiles = base[n_inst];
    b->item = kChunk;
    b->work_cap = size_t(b->total_tiles + b->total_points / kMinBatchItem + 1);
    cudaError_t e = cudaMalloc(&b->geoms, sizeof(TiledGeom) * n_inst);
    if (e == cudaSuccess) e = cudaMalloc(&b->offs, sizeof(int64_t*) * n_inst);
    if (e == cudaSuccess) e = cudaMalloc(&b->tile_base, sizeof(int64_t) * (n_inst + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->work, sizeof(WorkItem) * b->work_cap);
    if (e == cudaSuccess) e = cudaMalloc(&b->work_prefix, sizeof(int64_t) * size_t(b->total_tiles + 1));
    if (e == cudaSuccess)
        e = cudaMalloc(&b->scratch, scan_scratch_bytes(b->total_tiles) + size_t(b->total_tiles) * 4 + 1024);
    if (e == cudaSuccess) e = cudaMalloc(&b->flags, 64);
    if (e == cudaSuccess) e = cudaMemset(b->flags, 0, 64);
    if (e == cudaSuccess) e = cudaMemcpy(b->geoms, geoms.data(), sizeof(TiledGeom) * n_inst, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->offs, offs.data(), sizeof(int64_t*) * n_inst, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->tile_base, base.data(), sizeof(int64_t) * (n_inst + 1), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        batch_free(b);
        return cuda_fail(e, "cgx_batch_plan_create");
    }
    TiledParams& prm = b->prm;
    prm.instances = b->geoms;
    prm.num_point = b->total_points;
    prm.work = b->work;
    prm.work_count = reinterpret_cast<const int64_t*>(b->flags + 2);
    prm.work_counter = b->flags + 1;
    prm.error_flag = b->flags;
    // Prepare every kernel of the plan now, so executing it never touches
    // kernel attributes (and can be captured into a graph).
    int per_sm = 1 << 30;
    if (is_p2g) {
        b->box_bytes = size_t(prm.smem_floats) * sizeof(float);
        int p = 0;
        e = prepare_p2g_tiled(prm, spline_order, true, b->box_bytes, &p);
        per_sm = p;
    } else {
        b->slot_smem.resize(n_arrays);
        for (int a = 0; a < n_arrays && e == cudaSuccess; ++a) {
            TiledParams one = prm;
            one.arrays[a].smem_offset = 0;
            b->slot_smem[a] = g2p_tiled_smem(prm, a);
            int p = 0;
            e = prepare_g2p_tiled(one, spline_order, a, true, b->slot_smem[a], &p);
            per_sm = p < per_sm ? p : per_sm;
        }
    }
    if (e != cudaSuccess || per_sm < 1) {
        batch_free(b);
        return e != cudaSuccess ? cuda_fail(e, "cgx_batch_plan_create") : fail(CGX_ERR_NOT_SUPPORTED, "kernel cannot run");
    }
    b->max_per_sm = per_sm;
    b->ctas_per_sm = per_sm;
    *out = b;
    return CGX_OK;
}

cgx_status cgx_batch_plan_destroy(cgx_batch_plan plan) {
    batch_free(plan);
    return CGX_OK;
}

cgx_status cgx_batch_execute(cgx_batch_plan plan, unsigned flags, void* stream) {
    if (!plan) return fail(CGX_ERR_INVALID_ARG, "plan is NULL");
    return batch_run(plan, flags, reinterpret_cast<cudaStream_t>(stream));
}

cgx_status cgx_batch_get_config(cgx_batch_plan plan, int64_t* item_particles, int* ctas_per_sm) {
    if (!plan) return fail(CGX_ERR_INVALID_ARG, "plan is NULL");
    if (item_particles) *item_particles = plan->item;
    if (ctas_per_sm) *ctas_per_sm = plan->ctas_per_sm;
    return CGX_OK;
}

cgx_status cgx_batch_set_config(cgx_batch_plan plan, int64_t item_particles, int ctas_per_sm) {
    if (!plan) return fail(CGX_ERR_INVALID_ARG, "plan is NULL");
    const int64_t max_item = int64_t(1) << 20;
    if (item_particles < kMinBatchItem || item_particles > max_item)
        return fail(CGX_ERR_INVALID_ARG, "item_particles out of range");
    if (ctas_per_sm < 1 || ctas_per_sm > plan->max_per_sm)
        return fail(CGX_ERR_INVALID_ARG, "ctas_per_sm must be in [1, resident CTAs per SM]");
    plan->item = item_particles;
    plan->ctas_per_sm = ctas_per_sm;
    return CGX_OK;
}

cgx_status cgx_batch_autotune(cgx_batch_plan plan, void* stream, double* best_ms) {
    if (!plan) return fail(CGX_ERR_INVALID_ARG, "plan is NULL");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t items[] = {1024, 2048, 4096, 8192, 16384};
    cudaEvent_t e0, e1;
    CGX_CUDA(cudaEventCreate(&e0));
    cudaError_t ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaEventDestroy(e0);
        return cuda_fail(ce, "cudaEventCreate");
    }
    float best = -1.0f;
    int64_t best_item = plan->item;
    int best_ctas = plan->ctas_per_sm;
    cgx_status s = CGX_OK;
    for (int64_t item : items) {
        for (int c = 1; c <= plan->max_per_sm && s == CGX_OK; ++c) {
            plan->item = item;
            plan->ctas_per_sm = c;
            s = batch_run(plan, 0, st);  // warm-up (work list, caches)
            if (s) break;
            float total = 0.0f;
            for (int rep = 0; rep < 3 && s == CGX_OK; ++rep) {
                cudaEventRecord(e0, st);
                s = batch_run(plan, 0, st);
                cudaEventRecord(e1, st);
                ce = cudaEventSynchronize(e1);
                if (ce != cudaSuccess) s = cuda_fail(ce, "cudaEventSynchronize");
                float ms = 0.0f;
                if (s == CGX_OK) cudaEventElapsedTime(&ms, e0, e1);
                total += ms;
            }
            if (s == CGX_OK && (best < 0.0f || total < best)) {
                best = total;
                best_item = item;
                best_ctas = c;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    plan->item = best_item;
    plan->ctas_per_sm = best_ctas;
    if (best_ms) *best_ms = best < 0.0f ? 0.0 : double(best) / 3.0;
    return s;
}

}  // extern "C"
