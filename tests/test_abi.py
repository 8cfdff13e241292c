"""CPU checks of the C ABI: libcgx.so loads, exports every function declared
in include/cgx.h, the ctypes structures match the C layout, and host-only
entry points / argument checks behave (no GPU work is launched)."""
import ctypes
import os
import re
import subprocess

import pytest

from cabana_gb300 import _lib as L
from cabana_gb300 import mesh as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cgx.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cgx_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(L.LIB_PATH):
        pytest.fail("libcgx.so is not built (run __graft_entry__.build())")
    return L.lib()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert names, "no declarations parsed"
    assert sorted(L.EXPORTS) == names
    for n in names:
        assert hasattr(lib, n), n


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "cgx.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\\n", sizeof(cgx_mesh), sizeof(cgx_field), sizeof(cgx_array), sizeof(cgx_op), sizeof(cgx_tiling));
  printf("%zu %zu %zu %zu\\n", offsetof(cgx_mesh, owned_cells), offsetof(cgx_mesh, entity), offsetof(cgx_op, x), offsetof(cgx_op, array));
  printf("%zu %zu\\n", offsetof(cgx_field, soa_stride), offsetof(cgx_tiling, tile_offsets));
  printf("%zu %zu %zu %zu\\n", sizeof(cgx_adjoint_op), offsetof(cgx_adjoint_op, x_bar), offsetof(cgx_adjoint_op, array),
         offsetof(cgx_adjoint_op, array_bar));
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    got = list(map(int, out))
    want = [ctypes.sizeof(L.CgxMesh), ctypes.sizeof(L.CgxField), ctypes.sizeof(L.CgxArray), ctypes.sizeof(L.CgxOp),
            ctypes.sizeof(L.CgxTiling), L.CgxMesh.owned_cells.offset, L.CgxMesh.entity.offset, L.CgxOp.x.offset,
            L.CgxOp.array.offset, L.CgxField.soa_stride.offset, L.CgxTiling.tile_offsets.offset,
            ctypes.sizeof(L.CgxAdjointOp), L.CgxAdjointOp.x_bar.offset, L.CgxAdjointOp.array.offset,
            L.CgxAdjointOp.array_bar.offset]
    assert got == want


def test_host_only_entry_points(lib):
    assert lib.cgx_version().decode().startswith("cgx")
    d3 = ctypes.c_double * 3
    nb = (ctypes.c_int32 * 3)()
    assert lib.cgx_cartesian_num_bins(d3(0, 0, 0), d3(10, 10, 10), d3(1, 1, 1), nb) == 0
    assert tuple(nb) == (10, 10, 10)
    assert lib.cgx_cartesian_num_bins(d3(0, 0, 0), d3(1, 1, 1), d3(0.3, 0.3, 0.3), nb) == 0
    assert tuple(nb) == M.cartesian_num_bins((0, 0, 0), (1, 1, 1), (0.3, 0.3, 0.3))
    assert lib.cgx_cartesian_num_bins(d3(0, 0, 0), d3(1, 1, 1), d3(-1, 1, 1), nb) == L.CGX_ERR_INVALID_ARG

    _, mp = M.simple_mesh(20, 0.5, halo_width=1)
    t = L.CgxTiling()
    assert lib.cgx_tiling_init(ctypes.byref(L.make_mesh(mp)), 2, (ctypes.c_int32 * 3)(8, 8, 8), ctypes.byref(t)) == 0
    # base nodes of a quadratic stencil: 0 .. ext-3 -> 21 - 2 = 21 bases over 23 nodes
    assert tuple(t.num_tiles) == (3, 3, 3)
    assert lib.cgx_tiling_num_offsets(ctypes.byref(t)) == 28


def test_argument_checks_fail_loudly(lib):
    _, mp = M.simple_mesh(4)
    mesh = L.make_mesh(mp)
    pts = L.CgxField()
    ops = (L.CgxOp * 1)()
    # NULL handle
    st = lib.cgx_p2g(None, ctypes.byref(mesh), ctypes.byref(pts), 1, 1, ops, 1, 0, None, 0, None)
    assert st == L.CGX_ERR_INVALID_ARG
    assert b"handle" in lib.cgx_last_error()
    aops = (L.CgxAdjointOp * 1)()
    st = lib.cgx_p2g_adjoint(None, ctypes.byref(mesh), ctypes.byref(pts), 1, 1, aops, 1, 0, None, None, 0, None)
    assert st == L.CGX_ERR_INVALID_ARG
    assert b"handle" in lib.cgx_last_error()
    bad = L.CgxMesh()
    bad.cell_size[0] = -1.0
    t = L.CgxTiling()
    assert lib.cgx_tiling_init(ctypes.byref(bad), 2, (ctypes.c_int32 * 3)(8, 8, 8), ctypes.byref(t)) == L.CGX_ERR_INVALID_ARG
    assert lib.cgx_tiling_init(ctypes.byref(mesh), 9, (ctypes.c_int32 * 3)(8, 8, 8), ctypes.byref(t)) == L.CGX_ERR_NOT_SUPPORTED
    # 2D meshes: accepted by the interpolation entry points, refused by the
    # 3D-only tiling; other dimension counts are refused
    gm2 = M.createUniformGlobalMesh((0.0, 0.0), (2.0, 3.0), 0.5)
    mesh2 = L.make_mesh(M.mesh_params(M.createLocalGrid(M.createGlobalGrid(gm2), 1)))
    assert mesh2.num_space_dim == 2 and mesh2.owned_cells[2] == 1
    assert lib.cgx_tiling_init(ctypes.byref(mesh2), 2, (ctypes.c_int32 * 3)(8, 8, 8), ctypes.byref(t)) == L.CGX_ERR_NOT_SUPPORTED
    assert b"3D" in lib.cgx_last_error()
    mesh4 = L.make_mesh(mp)
    mesh4.num_space_dim = 4
    assert lib.cgx_tiling_init(ctypes.byref(mesh4), 2, (ctypes.c_int32 * 3)(8, 8, 8), ctypes.byref(t)) == L.CGX_ERR_INVALID_ARG
    d2 = ctypes.c_double * 2
    st = lib.cgx_linked_cell_build_2d(None, ctypes.byref(pts), 0, 1, d2(0, 0), d2(1, 1), d2(1, 1), None, None, None,
                                      None)
    assert st == L.CGX_ERR_INVALID_ARG
    assert b"handle" in lib.cgx_last_error()
    # binByKey / sortByKey: the handle is checked first, then the range and nbin
    st = lib.cgx_bin_by_key_range(None, None, 0, 4, 3, 0, None, None, None, None)
    assert st == L.CGX_ERR_INVALID_ARG and b"handle" in lib.cgx_last_error()


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No CPU fallback: without libcgx.so every entry point refuses to run."""
    monkeypatch.setattr(L, "_lib", None)
    monkeypatch.setattr(L, "LIB_PATH", str(tmp_path / "libcgx.so"))
    with pytest.raises(RuntimeError, match="missing"):
        L.lib()
