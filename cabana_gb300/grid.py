"""Cabana::Grid interpolation API over torch CUDA tensors.

Mirrors the reference's call shapes (grid/src/Cabana_Grid_Interpolation.hpp):

    p2g(functor, points, num_point, Spline(N), halo, array)
    g2p(array, halo, points, num_point, Spline(N), functor)

with the ten functor factories (createScalarValueP2G, ..., createVector
DivergenceG2P), Array / ArrayLayout / createArray, createHalo and
ArrayOp.assign. Every call goes through libcgx.so's C ABI; there is no
Python or PyTorch compute path. Beyond the reference signature, p2g / g2p
accept a list of functors (one launch, one spline evaluation) and the
keyword arguments `precision` and `tiling`.

Particle fields are torch tensors indexed (p), (p, d) or (p, m, n) in any
row-major layout, or `Slice` objects describing AoSoA members.
"""
import ctypes
from dataclasses import dataclass
from typing import Optional

import torch

from . import _lib as L
from . import mesh as M
from .mesh import (Cell, Node, createGlobalGrid, createLocalGrid, createLocalMesh,  # noqa: F401  (re-exported API)
                   createUniformGlobalMesh)

PLAIN_FP64 = L.CGX_PLAIN_FP64
FP32_COMPENSATED = L.CGX_FP32_COMPENSATED


class Own:
    """Decomposition tag (Cabana::Grid::Own)."""


class Ghost:
    """Decomposition tag (Cabana::Grid::Ghost)."""


@dataclass(frozen=True)
class Spline:
    """Cabana::Grid::Spline<order> tag."""
    order: int


class NodeHaloPattern:
    """NodeHaloPattern<3> (26 neighbours) or NodeHaloPattern<2> (8): on one
    rank both reduce to the periodic fold / fill of the mesh's dimensions."""


def _dtype_code(t):
    if t == torch.float64:
        return L.CGX_F64
    if t == torch.float32:
        return L.CGX_F32
    raise TypeError(f"unsupported dtype {t}; use float32 or float64")


@dataclass
class Slice:
    """A Cabana::Slice of an AoSoA member: `storage` is the flat tensor of the
    whole AoSoA (any dtype view of it), `offset` the element offset of member
    element (0, 0) inside it, `vector_length` the SoA width, `soa_stride` the
    number of member-type elements per SoA, `comps` the member's flattened
    extra extent (core/src/Cabana_Slice.hpp:96-190)."""
    storage: torch.Tensor
    offset: int
    vector_length: int
    soa_stride: int
    comps: int
    size: int

    def descriptor(self):
        f = L.CgxField()
        f.data = self.storage.data_ptr() + self.offset * self.storage.element_size()
        f.dtype = _dtype_code(self.storage.dtype)
        f.vector_length = self.vector_length
        f.soa_stride = self.soa_stride
        f.comp_stride = self.vector_length
        return f


def field_descriptor(x):
    """cgx_field for a tensor (p, ...) or a Slice."""
    if isinstance(x, Slice):
        return x.descriptor()
    if not isinstance(x, torch.Tensor):
        raise TypeError("particle fields must be torch tensors or Slice objects")
    if not x.is_cuda:
        raise ValueError("particle fields must live on the GPU")
    f = L.CgxField()
    f.data = x.data_ptr()
    f.dtype = _dtype_code(x.dtype)
    f.vector_length = 1
    f.soa_stride = x.stride(0)
    if x.dim() == 1:
        f.comp_stride = 1
    elif x.dim() == 2:
        f.comp_stride = x.stride(1)  # LayoutRight (p, d): 1; LayoutLeft: n
    else:
        # (p, m, n): the flattened component c = m * N + n must be one stride
        if x.stride(1) != x.shape[2] * x.stride(2):
            raise ValueError("a (p, m, n) field needs stride(1) == extent(2) * stride(2)")
        f.comp_stride = x.stride(2)
    return f


@dataclass
class ArrayLayout:
    local_grid: M.LocalGrid
    dofs: int
    entity: int

    def mesh_params(self):
        return M.mesh_params(self.local_grid, self.entity)


def createArrayLayout(local_grid, dofs_per_entity, entity=Node):
    ent = entity.value if hasattr(entity, "value") else int(entity)
    return ArrayLayout(local_grid, int(dofs_per_entity), ent)


class Array:
    """Cabana::Grid::Array: a (i, j, k, dof) tensor -- (i, j, dof) on a 2D
    mesh -- over the ghosted index space (grid/src/Cabana_Grid_Array.hpp:
    44-300)."""

    def __init__(self, label, layout: ArrayLayout, dtype=torch.float64, device="cuda", data=None):
        self.label = label
        self._layout = layout
        ext = layout.mesh_params().extents()
        if data is None:
            self._view = torch.zeros(ext + (layout.dofs,), dtype=dtype, device=device)
        else:
            # wrap existing contiguous storage (e.g. a slice of a pooled buffer)
            if tuple(data.shape) != ext + (layout.dofs,) or not data.is_contiguous():
                raise ValueError("data must be a contiguous (i, j, [k,] dof) tensor of the layout's extents")
            self._view = data

    def layout(self):
        return self._layout

    def view(self):
        return self._view

    def descriptor(self):
        a = L.CgxArray()
        a.data = self._view.data_ptr()
        a.dtype = _dtype_code(self._view.dtype)
        a.dofs = self._layout.dofs
        return a

    def mesh(self):
        return L.make_mesh(self._layout.mesh_params())


def createArray(label, layout, dtype=torch.float64, data=None):
    return Array(label, layout, dtype, data=data)


class Halo:
    """Grid halo for NodeHaloPattern<3> on one rank."""

    def __init__(self, width):
        self.width = width

    def gather(self, array: Array, stream=None):
        L.check(L.lib().cgx_halo_gather(ctypes.byref(array.mesh()), ctypes.byref(array.descriptor()),
                                        _stream(stream)))

    def scatter(self, array: Array, stream=None):
        L.check(L.lib().cgx_halo_scatter_sum(ctypes.byref(array.mesh()), ctypes.byref(array.descriptor()),
                                             _stream(stream)))


def createHalo(pattern, width, array=None):
    return Halo(width)


class ArrayOp:
    @staticmethod
    def assign(array: Array, value, decomposition=Ghost, stream=None):
        """ArrayOp::assign (grid/src/Cabana_Grid_Array.hpp:431-447)."""
        if decomposition is Ghost:
            L.check(L.lib().cgx_array_assign(ctypes.byref(array.mesh()), ctypes.byref(array.descriptor()),
                                             float(value), _stream(stream)))
        else:
            own = array.layout().local_grid.ownedSpace(array.layout().entity)
            array.view()[tuple(slice(a, b) for a, b in own)] = value


# ---- functors ----------------------------------------------------------

@dataclass
class Functor:
    kind: int
    x: object
    multiplier: float
    p2g: bool
    rank: int


def _mk(kind, x, multiplier, p2g, rank):
    if isinstance(x, torch.Tensor):
        got = x.dim()
        if got != rank:
            # the reference static_asserts on the View rank (Interpolation.hpp:958, :1008, ...)
            raise TypeError(f"field must be rank {rank}, got rank {got}")
    return Functor(kind, x, float(multiplier), p2g, rank)


def createScalarValueP2G(x, multiplier):
    return _mk(0, x, multiplier, True, 1)


def createVectorValueP2G(x, multiplier):
    return _mk(1, x, multiplier, True, 2)


def createScalarGradientP2G(x, multiplier):
    return _mk(2, x, multiplier, True, 1)


def createVectorDivergenceP2G(x, multiplier):
    return _mk(3, x, multiplier, True, 2)


def createTensorDivergenceP2G(x, multiplier):
    return _mk(4, x, multiplier, True, 3)


def createScalarValueG2P(x, multiplier):
    return _mk(0, x, multiplier, False, 1)


def createVectorValueG2P(x, multiplier):
    return _mk(1, x, multiplier, False, 2)


def createScalarGradientG2P(x, multiplier):
    return _mk(2, x, multiplier, False, 2)


def createVectorGradientG2P(x, multiplier):
    return _mk(3, x, multiplier, False, 3)


def createVectorDivergenceG2P(x, multiplier):
    return _mk(4, x, multiplier, False, 1)


def _stream(stream):
    if stream is None:
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, torch.cuda.Stream):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))


def _ops(functors, arrays):
    n = len(functors)
    ops = (L.CgxOp * n)()
    for i, (f, a) in enumerate(zip(functors, arrays)):
        ops[i].kind = f.kind
        ops[i].multiplier = f.multiplier
        ops[i].x = field_descriptor(f.x)
        ops[i].array = a.descriptor()
    return ops


def _as_list(v):
    return list(v) if isinstance(v, (list, tuple)) else [v]


def p2g(functor, points, num_point, spline: Spline, halo: Optional[Halo], array, *, precision=PLAIN_FP64,
        tiling=None, handle=None, stream=None, flags=0, check_bounds=False):
    """Cabana::Grid::p2g (grid/src/Cabana_Grid_Interpolation.hpp:1217-1313).

    `functor` / `array` may be lists of equal length: functor i scatters into
    array i, all in one launch. Contributions are added to the arrays; when
    `halo` is given the scatter(Sum) runs afterwards.
    """
    fs, arrs = _as_list(functor), _as_list(array)
    if len(arrs) == 1 and len(fs) > 1:
        arrs = arrs * len(fs)
    if any(not f.p2g for f in fs):
        raise TypeError("p2g needs P2G functors")
    mesh = arrs[0].mesh()
    ops = _ops(fs, arrs)
    pts = field_descriptor(points)
    h = handle or L.default_handle()
    fl = flags | (0 if halo is not None else L.CGX_FLAG_SKIP_HALO) | (L.CGX_FLAG_CHECK_BOUNDS if check_bounds else 0)
    til = ctypes.byref(tiling.struct) if tiling is not None else None
    L.check(L.lib().cgx_p2g(h.ptr, ctypes.byref(mesh), ctypes.byref(pts), int(num_point), spline.order, ops,
                            len(fs), precision, til, fl, _stream(stream)))


def g2p(array, halo: Optional[Halo], points, num_point, spline: Spline, functor, *, precision=PLAIN_FP64,
        tiling=None, handle=None, stream=None, flags=0, check_bounds=False):
    """Cabana::Grid::g2p (grid/src/Cabana_Grid_Interpolation.hpp:831-927)."""
    fs, arrs = _as_list(functor), _as_list(array)
    if len(arrs) == 1 and len(fs) > 1:
        arrs = arrs * len(fs)
    if any(f.p2g for f in fs):
        raise TypeError("g2p needs G2P functors")
    mesh = arrs[0].mesh()
    ops = _ops(fs, arrs)
    pts = field_descriptor(points)
    h = handle or L.default_handle()
    fl = flags | (0 if halo is not None else L.CGX_FLAG_SKIP_HALO) | (L.CGX_FLAG_CHECK_BOUNDS if check_bounds else 0)
    til = ctypes.byref(tiling.struct) if tiling is not None else None
    L.check(L.lib().cgx_g2p(h.ptr, ctypes.byref(mesh), ctypes.byref(pts), int(num_point), spline.order, ops,
                            len(fs), precision, til, fl, _stream(stream)))


def g2p2g(p2g_functor, points, num_point, spline: Spline, halo: Optional[Halo], p2g_array, g2p_functor,
          g2p_array=None, *, precision=PLAIN_FP64, tiling=None, handle=None, stream=None, flags=0,
          check_bounds=False):
    """Fused G2P then P2G per point, one spline evaluation (the g2p2g of
    benchmark/grid/Cabana_Grid_InterpolationPerformance.cpp:129-174, whose
    call shape `g2p2g(scalar_p2g, points, num_point, halo, array,
    scalar_g2p)` this follows, plus the spline tag).

    The G2P functors gather from `g2p_array` (default: `p2g_array`) into
    their point fields; the P2G functors then scatter into `p2g_array`. G2P
    reads each array as it was at the call (a snapshot where a P2G functor
    also writes it). Lists of functors and arrays are accepted as in p2g /
    g2p. With a `tiling` and the FP32 form the tiled G2P then P2G launches
    run (same results, faster); otherwise one fused point kernel.
    """
    pf, pa = _as_list(p2g_functor), _as_list(p2g_array)
    gf = _as_list(g2p_functor)
    ga = _as_list(g2p_array) if g2p_array is not None else pa
    if len(pa) == 1 and len(pf) > 1:
        pa = pa * len(pf)
    if len(ga) == 1 and len(gf) > 1:
        ga = ga * len(gf)
    if any(not f.p2g for f in pf) or any(f.p2g for f in gf):
        raise TypeError("g2p2g needs P2G functors first and G2P functors last")
    mesh = pa[0].mesh()
    pops = _ops(pf, pa)
    gops = _ops(gf, ga)
    pts = field_descriptor(points)
    h = handle or L.default_handle()
    fl = flags | (0 if halo is not None else L.CGX_FLAG_SKIP_HALO) | (L.CGX_FLAG_CHECK_BOUNDS if check_bounds else 0)
    til = ctypes.byref(tiling.struct) if tiling is not None else None
    L.check(L.lib().cgx_g2p2g(h.ptr, ctypes.byref(mesh), ctypes.byref(pts), int(num_point), spline.order, gops,
                              len(gf), pops, len(pf), precision, til, fl, _stream(stream)))


def createTensorDivergenceTransposedP2G(x, multiplier):
    """TensorDivergenceP2G of the transposed tensor (no reference
    counterpart): grid_m += sum_n dW/dx_n x[n][m]."""
    return _mk(L.CGX_TENSOR_DIVERGENCE_T_P2G, x, multiplier, True, 3)


def createVectorGradientTransposedG2P(x, multiplier):
    """VectorGradientG2P stored transposed (no reference counterpart):
    x[m][n] += multiplier * sum dW/dx_n f_m."""
    return _mk(L.CGX_VECTOR_GRADIENT_T_G2P, x, multiplier, False, 3)


def _null_field():
    return L.CgxField()


def _null_array():
    return L.CgxArray()


def _adjoint_call(fn, functors, points, num_point, spline, halo, xs, x_bars, arrays, array_bars, points_bar,
                  precision, tiling, handle, stream, check_bounds):
    n = len(functors)
    ops = (L.CgxAdjointOp * n)()
    for i, f in enumerate(functors):
        ops[i].kind = f.kind
        ops[i].multiplier = f.multiplier
        ops[i].x = field_descriptor(xs[i]) if xs[i] is not None else _null_field()
        ops[i].x_bar = field_descriptor(x_bars[i]) if x_bars[i] is not None else _null_field()
        ops[i].array = arrays[i].descriptor() if arrays[i] is not None else _null_array()
        ops[i].array_bar = array_bars[i].descriptor() if array_bars[i] is not None else _null_array()
    grid_ref = next(a for a in list(array_bars) + list(arrays) if a is not None)
    mesh = grid_ref.mesh()
    pts = field_descriptor(points)
    pb = ctypes.byref(field_descriptor(points_bar)) if points_bar is not None else None
    h = handle or L.default_handle()
    fl = (0 if halo is not None else L.CGX_FLAG_SKIP_HALO) | (L.CGX_FLAG_CHECK_BOUNDS if check_bounds else 0)
    til = ctypes.byref(tiling.struct) if tiling is not None else None
    L.check(fn(h.ptr, ctypes.byref(mesh), ctypes.byref(pts), int(num_point), spline.order, ops, n, precision, til, pb,
               fl, _stream(stream)))


def p2g_adjoint(functor, points, num_point, spline: Spline, halo: Optional[Halo], array_bar, *, x_bar=None,
                points_bar=None, precision=PLAIN_FP64, tiling=None, handle=None, stream=None, check_bounds=False):
    """Reverse mode of p2g (no reference counterpart).

    `functor`: the forward P2G functors; `array_bar`: dL/d(forward array) per
    functor (read; its ghosts are halo-adjusted in place on periodic meshes
    when `halo` is given); `x_bar`: tensors receiving dL/d(functor field),
    added (entries may be None); `points_bar`: (n, 3) tensor receiving
    dL/d(position), added.
    """
    fs, abars = _as_list(functor), _as_list(array_bar)
    if len(abars) == 1 and len(fs) > 1:
        abars = abars * len(fs)
    if any(not f.p2g for f in fs):
        raise TypeError("p2g_adjoint needs P2G functors")
    xb = _as_list(x_bar) if x_bar is not None else [None] * len(fs)
    _adjoint_call(L.lib().cgx_p2g_adjoint, fs, points, num_point, spline, halo, [f.x for f in fs], xb,
                  [None] * len(fs), abars, points_bar, precision, tiling, handle, stream, check_bounds)


def g2p_adjoint(array, halo: Optional[Halo], points, num_point, spline: Spline, functor, x_bar, *, array_bar=None,
                points_bar=None, precision=PLAIN_FP64, tiling=None, handle=None, stream=None, check_bounds=False):
    """Reverse mode of g2p (no reference counterpart).

    `array`: the forward arrays as g2p read them; `functor`: the forward G2P
    functors; `x_bar`: dL/d(functor output field) per functor (read);
    `array_bar`: Arrays receiving dL/d(array), added (entries may be None);
    `points_bar`: (n, 3) tensor receiving dL/d(position), added.
    """
    fs, arrs = _as_list(functor), _as_list(array)
    if len(arrs) == 1 and len(fs) > 1:
        arrs = arrs * len(fs)
    if any(f.p2g for f in fs):
        raise TypeError("g2p_adjoint needs G2P functors")
    xb = _as_list(x_bar)
    ab = _as_list(array_bar) if array_bar is not None else [None] * len(fs)
    if len(ab) == 1 and len(fs) > 1:
        ab = ab * len(fs)
    _adjoint_call(L.lib().cgx_g2p_adjoint, fs, points, num_point, spline, halo, [None] * len(fs), xb,
                  arrs, ab, points_bar, precision, tiling, handle, stream, check_bounds)


@dataclass
class BatchInstance:
    """One independent problem of a batch: its points (tile-sorted with
    `tiling`), point count, and per-functor point field and Array."""
    points: object
    num_point: int
    tiling: "Tiling"
    fields: list
    arrays: list


class BatchPlan:
    """Batched p2g (p2g=True) or g2p over many meshes with one work list and
    one persistent launch (no reference counterpart). `functors` give the
    operator kinds and multipliers (their fields are ignored); each instance
    brings its own fields and arrays. execute() neither allocates nor
    synchronises, so it can be captured into a CUDA graph."""

    def __init__(self, functors, instances, spline: Spline, p2g=True, handle=None):
        fs = _as_list(functors)
        if any(f.p2g != p2g for f in fs):
            raise TypeError("functor direction does not match the plan")
        self._keep = list(instances)
        n = len(instances)
        inst = (L.CgxInstance * n)()
        for i, b in enumerate(instances):
            if len(b.fields) != len(fs) or len(b.arrays) != len(fs):
                raise ValueError("each instance needs one field and one array per functor")
            inst[i].mesh = b.arrays[0].mesh()
            inst[i].points = field_descriptor(b.points)
            inst[i].num_point = int(b.num_point)
            inst[i].tiling = b.tiling.struct
            for o in range(len(fs)):
                inst[i].x[o] = field_descriptor(b.fields[o])
                inst[i].array[o] = b.arrays[o].descriptor()
        ops = (L.CgxOp * len(fs))()
        for o, f in enumerate(fs):
            ops[o].kind = f.kind
            ops[o].multiplier = f.multiplier
        self._handle = handle or L.default_handle()
        plan = ctypes.c_void_p()
        L.check(L.lib().cgx_batch_plan_create(self._handle.ptr, inst, n, spline.order, ops, len(fs), int(bool(p2g)),
                                              ctypes.byref(plan)))
        self.ptr = plan

    def execute(self, stream=None, halo=True, check_bounds=False):
        fl = (0 if halo else L.CGX_FLAG_SKIP_HALO) | (L.CGX_FLAG_CHECK_BOUNDS if check_bounds else 0)
        L.check(L.lib().cgx_batch_execute(self.ptr, fl, _stream(stream)))

    def autotune(self, stream=None):
        best = ctypes.c_double()
        L.check(L.lib().cgx_batch_autotune(self.ptr, _stream(stream), ctypes.byref(best)))
        return best.value

    def config(self):
        item = ctypes.c_int64()
        ctas = ctypes.c_int()
        L.check(L.lib().cgx_batch_get_config(self.ptr, ctypes.byref(item), ctypes.byref(ctas)))
        return item.value, ctas.value

    def set_config(self, item_particles, ctas_per_sm):
        L.check(L.lib().cgx_batch_set_config(self.ptr, int(item_particles), int(ctas_per_sm)))

    def __del__(self):
        try:
            if getattr(self, "ptr", None):
                L.lib().cgx_batch_plan_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass


def last_dispatch(handle=None):
    """Kernel family of the last p2g / g2p on the handle: 'points' or 'tiled'."""
    h = handle or L.default_handle()
    return {L.CGX_DISPATCH_NONE: None, L.CGX_DISPATCH_POINTS: "points",
            L.CGX_DISPATCH_TILED: "tiled"}[L.lib().cgx_last_dispatch(h.ptr)]


class Tiling:
    """Tile-major ordering of particles for the tiled kernels."""

    def __init__(self, mesh_params, order, tile=(8, 8, 8), device="cuda"):
        self.struct = L.CgxTiling()
        t = (ctypes.c_int32 * 3)(*tile)
        L.check(L.lib().cgx_tiling_init(ctypes.byref(L.make_mesh(mesh_params)), order, t, ctypes.byref(self.struct)))
        n = L.lib().cgx_tiling_num_offsets(ctypes.byref(self.struct))
        self.offsets = torch.zeros(n, dtype=torch.int64, device=device)
        self.struct.tile_offsets = self.offsets.data_ptr()
        self.mesh_params = mesh_params
        self.order = order

    def sort(self, points, num_point, handle=None, stream=None):
        """Compute the tile-major gather permutation of `points` (uint64 as int64)."""
        perm = torch.empty(max(1, num_point), dtype=torch.int64, device=self.offsets.device)
        h = handle or L.default_handle()
        L.check(L.lib().cgx_sort_tiles(h.ptr, ctypes.byref(L.make_mesh(self.mesh_params)),
                                       ctypes.byref(field_descriptor(points)), int(num_point),
                                       ctypes.byref(self.struct), ctypes.c_void_p(perm.data_ptr()), _stream(stream)))
        return perm[:num_point]
