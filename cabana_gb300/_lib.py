"""ctypes binding of libcgx.so (the C ABI declared in include/cgx.h).

The library is loaded from this package directory. There is no fallback:
if libcgx.so is missing or fails to load, every call raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcgx.so")

CGX_OK = 0
CGX_ERR_INVALID_ARG = 1
CGX_ERR_CUDA = 2
CGX_ERR_OUT_OF_BOUNDS = 3
CGX_ERR_TIMEOUT = 4
CGX_ERR_NOT_SUPPORTED = 5
CGX_ERR_NO_MEMORY = 6

CGX_F32 = 0
CGX_F64 = 1
CGX_NODE = 0
CGX_CELL = 1
CGX_PLAIN_FP64 = 0
CGX_FP32_COMPENSATED = 1

# transposed tensor operators (no reference counterpart; used by the adjoints)
CGX_TENSOR_DIVERGENCE_T_P2G = 5
CGX_VECTOR_GRADIENT_T_G2P = 5

CGX_FLAG_SKIP_HALO = 1
CGX_FLAG_CHECK_BOUNDS = 2

# Every exported symbol declared in include/cgx.h.
CGX_DISPATCH_NONE = 0
CGX_DISPATCH_POINTS = 1
CGX_DISPATCH_TILED = 2

EXPORTS = (
    "cgx_create", "cgx_destroy", "cgx_last_error", "cgx_version", "cgx_last_dispatch",
    "cgx_p2g", "cgx_g2p", "cgx_g2p2g", "cgx_p2g_adjoint", "cgx_g2p_adjoint", "cgx_halo_scatter_sum", "cgx_halo_gather", "cgx_array_assign",
    "cgx_cartesian_num_bins", "cgx_linked_cell_build", "cgx_linked_cell_build_2d", "cgx_bin_by_key", "cgx_bin_by_key_range", "cgx_bin_by_key_static", "cgx_permute",
    "cgx_tiling_init", "cgx_tiling_num_offsets", "cgx_sort_tiles",
    "cgx_batch_plan_create", "cgx_batch_plan_destroy", "cgx_batch_execute", "cgx_batch_autotune",
    "cgx_batch_get_config", "cgx_batch_set_config",
)


class CgxMesh(ctypes.Structure):
    _fields_ = [
        ("ghost_low", ctypes.c_double * 3),
        ("cell_size", ctypes.c_double * 3),
        ("owned_cells", ctypes.c_int32 * 3),
        ("halo_width", ctypes.c_int32),
        ("periodic", ctypes.c_int32 * 3),
        ("entity", ctypes.c_int32),
        ("num_space_dim", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class CgxField(ctypes.Structure):
    _fields_ = [
        ("data", ctypes.c_void_p),
        ("dtype", ctypes.c_int32),
        ("vector_length", ctypes.c_int32),
        ("soa_stride", ctypes.c_int64),
        ("comp_stride", ctypes.c_int64),
    ]


class CgxArray(ctypes.Structure):
    _fields_ = [
        ("data", ctypes.c_void_p),
        ("dtype", ctypes.c_int32),
        ("dofs", ctypes.c_int32),
    ]


class CgxOp(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("multiplier", ctypes.c_double),
        ("x", CgxField),
        ("array", CgxArray),
    ]


class CgxAdjointOp(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("multiplier", ctypes.c_double),
        ("x", CgxField),
        ("x_bar", CgxField),
        ("array", CgxArray),
        ("array_bar", CgxArray),
    ]


class CgxTiling(ctypes.Structure):
    _fields_ = [
        ("tile", ctypes.c_int32 * 3),
        ("num_tiles", ctypes.c_int32 * 3),
        ("spline_order", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("tile_offsets", ctypes.c_void_p),
    ]


CGX_BATCH_MAX_OPS = 8


class CgxInstance(ctypes.Structure):
    _fields_ = [
        ("mesh", CgxMesh),
        ("points", CgxField),
        ("num_point", ctypes.c_int64),
        ("tiling", CgxTiling),
        ("x", CgxField * CGX_BATCH_MAX_OPS),
        ("array", CgxArray * CGX_BATCH_MAX_OPS),
    ]


class CgxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cgx error {code}: {msg}")
        self.code = code


_lib = None


def lib():
    """Load libcgx.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() (or python cabana_gb300/build.py)")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    L.cgx_create.argtypes = [P(vp)]
    L.cgx_destroy.argtypes = [vp]
    L.cgx_last_error.restype = ctypes.c_char_p
    L.cgx_version.restype = ctypes.c_char_p
    L.cgx_last_dispatch.argtypes = [vp]
    L.cgx_last_dispatch.restype = ctypes.c_int
    interp = [vp, P(CgxMesh), P(CgxField), ctypes.c_int64, ctypes.c_int, P(CgxOp), ctypes.c_int, ctypes.c_int,
              P(CgxTiling), ctypes.c_uint, vp]
    L.cgx_p2g.argtypes = interp
    L.cgx_g2p.argtypes = interp
    L.cgx_g2p2g.argtypes = [vp, P(CgxMesh), P(CgxField), ctypes.c_int64, ctypes.c_int, P(CgxOp), ctypes.c_int, P(CgxOp),
                            ctypes.c_int, ctypes.c_int, P(CgxTiling), ctypes.c_uint, vp]
    adj = [vp, P(CgxMesh), P(CgxField), ctypes.c_int64, ctypes.c_int, P(CgxAdjointOp), ctypes.c_int, ctypes.c_int,
           P(CgxTiling), P(CgxField), ctypes.c_uint, vp]
    L.cgx_p2g_adjoint.argtypes = adj
    L.cgx_g2p_adjoint.argtypes = adj
    L.cgx_batch_plan_create.argtypes = [vp, P(CgxInstance), ctypes.c_int, ctypes.c_int, P(CgxOp), ctypes.c_int,
                                        ctypes.c_int, P(vp)]
    L.cgx_batch_plan_destroy.argtypes = [vp]
    L.cgx_batch_execute.argtypes = [vp, ctypes.c_uint, vp]
    L.cgx_batch_autotune.argtypes = [vp, vp, P(ctypes.c_double)]
    L.cgx_batch_get_config.argtypes = [vp, P(ctypes.c_int64), P(ctypes.c_int)]
    L.cgx_batch_set_config.argtypes = [vp, ctypes.c_int64, ctypes.c_int]
    L.cgx_halo_scatter_sum.argtypes = [P(CgxMesh), P(CgxArray), vp]
    L.cgx_halo_gather.argtypes = [P(CgxMesh), P(CgxArray), vp]
    L.cgx_array_assign.argtypes = [P(CgxMesh), P(CgxArray), ctypes.c_double, vp]
    d3 = ctypes.c_double * 3
    L.cgx_cartesian_num_bins.argtypes = [d3, d3, d3, ctypes.c_int32 * 3]
    L.cgx_linked_cell_build.argtypes = [vp, P(CgxField), ctypes.c_int64, ctypes.c_int64, d3, d3, d3, vp, vp, vp, vp]
    d2 = ctypes.c_double * 2
    L.cgx_linked_cell_build_2d.argtypes = [vp, P(CgxField), ctypes.c_int64, ctypes.c_int64, d2, d2, d2, vp, vp, vp,
                                           vp]
    L.cgx_bin_by_key.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, vp, vp, vp, vp]
    L.cgx_bin_by_key_range.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int, vp, vp,
                                        vp, vp]
    L.cgx_bin_by_key_static.argtypes = [vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, vp, vp, vp, vp]
    L.cgx_permute.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_int64, P(CgxField), P(ctypes.c_int32), ctypes.c_int, vp]
    L.cgx_tiling_init.argtypes = [P(CgxMesh), ctypes.c_int, ctypes.c_int32 * 3, P(CgxTiling)]
    L.cgx_tiling_num_offsets.argtypes = [P(CgxTiling)]
    L.cgx_tiling_num_offsets.restype = ctypes.c_int64
    L.cgx_sort_tiles.argtypes = [vp, P(CgxMesh), P(CgxField), ctypes.c_int64, P(CgxTiling), vp, vp]
    _lib = L
    return L


def check(status):
    if status != CGX_OK:
        raise CgxError(status, lib().cgx_last_error().decode())
    return status


def make_mesh(params):
    """CgxMesh from a cabana_gb300.mesh.MeshParams (3D or 2D)."""
    m = CgxMesh()
    nd = getattr(params, "num_space_dim", 3)
    for d in range(3):
        m.ghost_low[d] = params.ghost_low[d] if d < nd else 0.0
        m.cell_size[d] = params.cell_size[d] if d < nd else 1.0
        m.owned_cells[d] = params.owned_cells[d] if d < nd else 1
        m.periodic[d] = params.periodic[d] if d < nd else 0
    m.halo_width = params.halo_width
    m.entity = params.entity
    m.num_space_dim = nd
    return m


class Handle:
    """Owns one cgx_handle (workspace, error flags)."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().cgx_create(ctypes.byref(h)))
        self.ptr = h

    def __del__(self):
        try:
            if self.ptr:
                lib().cgx_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass


_default = None


def default_handle():
    global _default
    if _default is None:
        _default = Handle()
    return _default
