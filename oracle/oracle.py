"""ctypes front end of the FP64 CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``. The product path never imports
this module.

Arrays are plain numpy float64 arrays: points ``(n, 3)``, particle fields
``(n, comps)`` and grid arrays ``(ni, nj, nk, dofs)`` in C order, which is the
reference's LayoutRight ``Array`` layout. On a 2D mesh (``make_mesh(...,
num_space_dim=2)``) points are ``(n, 2)``, vectors have 2 components, tensors
4, and grid arrays are ``(ni, nj, dofs)``.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

# kind 5 is the transposed tensor form (no reference counterpart) used by the adjoints
P2G_COMPS = {0: 1, 1: 3, 2: 1, 3: 3, 4: 9, 5: 9}
P2G_DOFS = {0: 1, 1: 3, 2: 3, 3: 1, 4: 3, 5: 3}
G2P_COMPS = {0: 1, 1: 3, 2: 3, 3: 9, 4: 1, 5: 9}
G2P_DOFS = {0: 1, 1: 3, 2: 1, 3: 3, 4: 3, 5: 3}
P2G_COMPS_2D = {0: 1, 1: 2, 2: 1, 3: 2, 4: 4, 5: 4}
P2G_DOFS_2D = {0: 1, 1: 2, 2: 2, 3: 1, 4: 2, 5: 2}
G2P_COMPS_2D = {0: 1, 1: 2, 2: 2, 3: 4, 4: 1, 5: 4}
G2P_DOFS_2D = {0: 1, 1: 2, 2: 1, 3: 2, 4: 2, 5: 2}


class OracleMesh(ctypes.Structure):
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


class OracleOp(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("dofs", ctypes.c_int32),
        ("multiplier", ctypes.c_double),
        ("x", ctypes.POINTER(ctypes.c_double)),
        ("array", ctypes.POINTER(ctypes.c_double)),
    ]


class OracleAdjointOp(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("dofs", ctypes.c_int32),
        ("multiplier", ctypes.c_double),
        ("x", ctypes.POINTER(ctypes.c_double)),
        ("x_bar", ctypes.POINTER(ctypes.c_double)),
        ("array", ctypes.POINTER(ctypes.c_double)),
        ("array_bar", ctypes.POINTER(ctypes.c_double)),
    ]


def build():
    """Compile the oracle with its Makefile (g++, no GPU needed)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        _lib.oracle_spline_map.restype = ctypes.c_double
        _lib.oracle_spline_map.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        _lib.oracle_spline_value.argtypes = [ctypes.c_int, ctypes.c_double, dp]
        _lib.oracle_spline_gradient.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, dp]
        _lib.oracle_spline_stencil.argtypes = [ctypes.c_int, ctypes.c_double, ip]
        _lib.oracle_spline_offsets.argtypes = [ctypes.c_int, ip]
        _lib.oracle_p2g.argtypes = [ctypes.POINTER(OracleMesh), dp, ctypes.c_int64, ctypes.c_int,
                                    ctypes.POINTER(OracleOp), ctypes.c_int, ctypes.c_int]
        _lib.oracle_g2p.argtypes = _lib.oracle_p2g.argtypes
        _lib.oracle_g2p2g.argtypes = [ctypes.POINTER(OracleMesh), dp, ctypes.c_int64, ctypes.c_int,
                                      ctypes.POINTER(OracleOp), ctypes.c_int, ctypes.POINTER(OracleOp), ctypes.c_int]
        _lib.oracle_spline_hessian.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, dp]
        _lib.oracle_p2g_adjoint.argtypes = [ctypes.POINTER(OracleMesh), dp, ctypes.c_int64, ctypes.c_int,
                                            ctypes.POINTER(OracleAdjointOp), ctypes.c_int, dp]
        _lib.oracle_g2p_adjoint.argtypes = _lib.oracle_p2g_adjoint.argtypes
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def make_mesh(ghost_low, cell_size, owned_cells, halo_width, periodic=(0, 0, 0), entity=0, num_space_dim=3):
    """Per-dimension arguments have num_space_dim entries (3 or 2)."""
    m = OracleMesh()
    for d in range(num_space_dim):
        m.ghost_low[d] = float(ghost_low[d])
        m.cell_size[d] = float(cell_size[d])
        m.owned_cells[d] = int(owned_cells[d])
        m.periodic[d] = int(bool(periodic[d]))
    for d in range(num_space_dim, 3):
        m.cell_size[d] = 1.0
        m.owned_cells[d] = 1
    m.halo_width = int(halo_width)
    m.entity = int(entity)
    m.num_space_dim = int(num_space_dim)
    return m


def extents(mesh):
    """Ghosted entity extents: 3 values, or 2 on a 2D mesh."""
    ext = np.zeros(3, np.int64)
    lib().oracle_extents(ctypes.byref(mesh), ext.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    return tuple(int(e) for e in ext[:2 if mesh.num_space_dim == 2 else 3])


def num_knot(order):
    return order + 1


def spline_map(order, xp, rdx, low_x):
    return lib().oracle_spline_map(order, xp, rdx, low_x)


def spline_value(order, x0):
    v = np.zeros(num_knot(order))
    lib().oracle_spline_value(order, x0, _dp(v))
    return v


def spline_gradient(order, x0, rdx):
    v = np.zeros(num_knot(order))
    lib().oracle_spline_gradient(order, x0, rdx, _dp(v))
    return v


def spline_hessian(order, x0, rdx):
    v = np.zeros(num_knot(order))
    lib().oracle_spline_hessian(order, x0, rdx, _dp(v))
    return v


def spline_stencil(order, x0):
    v = np.zeros(num_knot(order), np.int32)
    lib().oracle_spline_stencil(order, x0, _ip(v))
    return v


def spline_offsets(order):
    v = np.zeros(num_knot(order), np.int32)
    lib().oracle_spline_offsets(order, _ip(v))
    return v


def evaluate_spline(mesh, order, p):
    nk = num_knot(order)
    p = np.ascontiguousarray(p, np.float64)
    dx = np.zeros(3)
    x = np.zeros(3)
    s = np.zeros((3, nk), np.int32)
    w = np.zeros((3, nk))
    g = np.zeros((3, nk))
    d = np.zeros((3, nk))
    lib().oracle_evaluate_spline(ctypes.byref(mesh), order, _dp(p), _dp(dx), _dp(x), _ip(s), _dp(w), _dp(g), _dp(d))
    return dict(dx=dx, x=x, s=s, w=w, g=g, d=d)


def _ops(ops, n, comps_table):
    arr = (OracleOp * max(1, len(ops)))()
    keep = []
    for i, (kind, mult, x, array) in enumerate(ops):
        assert x.dtype == np.float64 and x.flags.c_contiguous
        assert array.dtype == np.float64 and array.flags.c_contiguous
        assert x.reshape(n, -1).shape[1] == comps_table[kind]
        arr[i].kind = kind
        arr[i].dofs = array.shape[-1]
        arr[i].multiplier = float(mult)
        arr[i].x = _dp(x)
        arr[i].array = _dp(array)
        keep.append((x, array))
    return arr, keep


def p2g(mesh, points, order, ops, nthreads=1):
    """ops: list of (kind, multiplier, x, array); arrays are updated in place."""
    points = np.ascontiguousarray(points, np.float64)
    n = points.shape[0]
    arr, _keep = _ops(ops, n, P2G_COMPS_2D if mesh.num_space_dim == 2 else P2G_COMPS)
    return lib().oracle_p2g(ctypes.byref(mesh), _dp(points), n, order, arr, len(ops), nthreads)


def g2p(mesh, points, order, ops, nthreads=1):
    """ops: list of (kind, multiplier, x, array); particle fields x are updated in place."""
    points = np.ascontiguousarray(points, np.float64)
    n = points.shape[0]
    arr, _keep = _ops(ops, n, G2P_COMPS_2D if mesh.num_space_dim == 2 else G2P_COMPS)
    return lib().oracle_g2p(ctypes.byref(mesh), _dp(points), n, order, arr, len(ops), nthreads)


def g2p2g(mesh, points, order, g2p_ops, p2g_ops):
    """Fused g2p2g. g2p_ops / p2g_ops: lists of (kind, multiplier, x, array);
    point fields and P2G arrays are updated in place; G2P reads each array as
    it was at the call (its ghosts are gathered in place first)."""
    points = np.ascontiguousarray(points, np.float64)
    n = points.shape[0]
    garr, _k1 = _ops(g2p_ops, n, G2P_COMPS)
    parr, _k2 = _ops(p2g_ops, n, P2G_COMPS)
    return lib().oracle_g2p2g(ctypes.byref(mesh), _dp(points), n, order, garr, len(g2p_ops), parr, len(p2g_ops))


def _adjoint(fn, mesh, points, order, ops, points_bar):
    points = np.ascontiguousarray(points, np.float64)
    n = points.shape[0]
    arr = (OracleAdjointOp * max(1, len(ops)))()
    null = ctypes.POINTER(ctypes.c_double)()
    for i, op in enumerate(ops):
        for key in ("x", "x_bar", "array", "array_bar"):
            a = op.get(key)
            assert a is None or (a.dtype == np.float64 and a.flags.c_contiguous), key
        grid = op.get("array_bar") if op.get("array_bar") is not None else op.get("array")
        arr[i].kind = op["kind"]
        arr[i].dofs = grid.shape[3]
        arr[i].multiplier = float(op["mult"])
        for key in ("x", "x_bar", "array", "array_bar"):
            setattr(arr[i], key, _dp(op[key]) if op.get(key) is not None else null)
    pb = _dp(points_bar) if points_bar is not None else null
    return fn(ctypes.byref(mesh), _dp(points), n, order, arr, len(ops), pb)


def p2g_adjoint(mesh, points, order, ops, points_bar=None):
    """Reverse mode of p2g. ops: dicts with kind, mult, x (forward input or
    None), x_bar (dL/dx, added, or None), array_bar (dL/d array, read; its
    ghosts are halo-adjusted in place on periodic meshes). points_bar (n, 3)
    receives dL/d(position), added."""
    return _adjoint(lib().oracle_p2g_adjoint, mesh, points, order, ops, points_bar)


def g2p_adjoint(mesh, points, order, ops, points_bar=None):
    """Reverse mode of g2p. ops: dicts with kind, mult, x_bar (dL/d output,
    read), array (forward array or None), array_bar (dL/d array, added, or
    None). points_bar (n, 3) receives dL/d(position), added."""
    return _adjoint(lib().oracle_g2p_adjoint, mesh, points, order, ops, points_bar)


def halo_scatter_sum(mesh, array):
    lib().oracle_halo_scatter_sum(ctypes.byref(mesh), _dp(array), ctypes.c_int(array.shape[-1]))


def halo_gather(mesh, array):
    lib().oracle_halo_gather(ctypes.byref(mesh), _dp(array), ctypes.c_int(array.shape[-1]))


def cartesian_num_bins(grid_min, grid_max, grid_delta):
    mn, mx, dl = (np.ascontiguousarray(v, np.float64) for v in (grid_min, grid_max, grid_delta))
    nb = np.zeros(3, np.int32)
    lib().oracle_cartesian_num_bins(_dp(mn), _dp(mx), _dp(dl), nb.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    return nb


def linked_cell_build(positions, begin, end, grid_min, grid_max, grid_delta):
    """LinkedCellList<..., nd>::build with nd = len(grid_min) (2 or 3);
    positions are (n, nd). Returns (nbin[nd], counts, offsets, permutes)."""
    mn, mx, dl = (np.ascontiguousarray(v, np.float64) for v in (grid_min, grid_max, grid_delta))
    nd = mn.shape[0]
    assert nd in (2, 3) and mx.shape[0] == nd and dl.shape[0] == nd
    positions = np.ascontiguousarray(positions, np.float64).reshape(-1, nd)
    nb = np.floor((mx - mn) * (1.0 / dl)).astype(np.int32) if nd == 2 else cartesian_num_bins(mn, mx, dl)
    ncell = int(np.prod(nb.astype(np.int64)))
    counts = np.zeros(ncell, np.int32)
    offsets = np.zeros(ncell, np.uint64)
    permutes = np.zeros(end - begin, np.uint64)
    u64 = ctypes.POINTER(ctypes.c_uint64)
    lib().oracle_linked_cell_build_nd(ctypes.c_int(nd), _dp(positions), ctypes.c_int64(begin), ctypes.c_int64(end),
                                      _dp(mn), _dp(mx), _dp(dl),
                                      counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                      offsets.ctypes.data_as(u64), permutes.ctypes.data_as(u64))
    return nb, counts, offsets, permutes


def bin_by_key_range(keys, nbin, begin=0, end=None, sort_within_bins=False):
    """Cabana::binByKey (sort_within_bins False) / sortByKey (True, with nbin =
    (end - begin) // 2) over int keys: nbin + 1 Kokkos::BinOp1D bins over the
    keys' [min, max]. Returns (counts, offsets, permutes)."""
    keys = np.ascontiguousarray(keys, np.int32)
    end = keys.shape[0] if end is None else end
    counts = np.zeros(nbin + 1, np.int32)
    offsets = np.zeros(nbin + 1, np.uint64)
    permutes = np.zeros(end - begin, np.uint64)
    u64 = ctypes.POINTER(ctypes.c_uint64)
    lib().oracle_bin_by_key_range(keys.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.c_int64(begin),
                                  ctypes.c_int64(end), ctypes.c_int32(nbin), ctypes.c_int(1 if sort_within_bins else 0),
                                  counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), offsets.ctypes.data_as(u64),
                                  permutes.ctypes.data_as(u64))
    return counts, offsets, permutes


def bin_by_key(keys, nbin, begin=0, end=None):
    keys = np.ascontiguousarray(keys, np.int32)
    end = keys.shape[0] if end is None else end
    counts = np.zeros(nbin, np.int32)
    offsets = np.zeros(nbin, np.uint64)
    permutes = np.zeros(end - begin, np.uint64)
    u64 = ctypes.POINTER(ctypes.c_uint64)
    lib().oracle_bin_by_key(keys.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.c_int64(begin),
                            ctypes.c_int64(end), ctypes.c_int32(nbin),
                            counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), offsets.ctypes.data_as(u64),
                            permutes.ctypes.data_as(u64))
    return counts, offsets, permutes


def permute(permutes, begin, end, data):
    """In-place permute of a (n, comps) float64 array over [begin, end)."""
    assert data.dtype == np.float64 and data.flags.c_contiguous
    comps = 1 if data.ndim == 1 else int(np.prod(data.shape[1:]))
    permutes = np.ascontiguousarray(permutes, np.uint64)
    lib().oracle_permute(permutes.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), ctypes.c_int64(begin),
                         ctypes.c_int64(end), _dp(data), ctypes.c_int(comps))


def stable_sort_keys(keys):
    keys = np.ascontiguousarray(keys, np.uint64)
    perm = np.zeros(keys.shape[0], np.uint64)
    u64 = ctypes.POINTER(ctypes.c_uint64)
    lib().oracle_stable_sort_keys(keys.ctypes.data_as(u64), ctypes.c_int64(keys.shape[0]), perm.ctypes.data_as(u64))
    return perm
