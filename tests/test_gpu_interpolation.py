"""GPU parity of p2g / g2p against the FP64 oracle, through the C ABI.

Tolerances (max|gpu - oracle| / max|oracle| over the whole output):
  * CGX_PLAIN_FP64:        1e-12 (atomic summation order only)
  * CGX_FP32_COMPENSATED:  P2G grid 1e-6, G2P point fields 2e-6
"""
import numpy as np
import pytest
import torch

from cabana_gb300 import grid as G
from cabana_gb300 import mesh as M
from tests.helpers import (G2P_COMPS, G2P_DOFS, P2G_COMPS, P2G_DOFS, clumped_points, domain, max_rel, oracle_mesh,
                           uniform_points)

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_P2G_FP32 = 1e-6      # tiled, compensated
TOL_P2G_FP32_POINTS = 4e-6  # point-parallel FP32 fallback: plain float atomics
TOL_G2P_FP32 = 2e-6

FORMS = [("plain64", G.PLAIN_FP64, False), ("fp32", G.FP32_COMPENSATED, False), ("fp32_tiled", G.FP32_COMPENSATED, True)]


def small_mesh(periodic=(False, False, False), halo=3, entity=M.NODE):
    gm = M.createUniformGlobalMesh((-1.3, 2.1, 0.4), (-1.3 + 12 * 0.37, 2.1 + 10 * 0.37, 0.4 + 9 * 0.37), 0.37)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, periodic), halo)
    return lg, M.mesh_params(lg, entity)


def layout(lg, dofs, entity=M.NODE):
    return G.createArrayLayout(lg, dofs, M.Node if entity == M.NODE else M.Cell)


def run_tolerance(form):
    return TOL_FP64 if form == G.PLAIN_FP64 else None


def sorted_inputs(mp, order, pts, fields, tiled):
    """Returns (points, fields, tiling) on the GPU, tile-sorted when asked."""
    tp = torch.tensor(pts, device="cuda")
    tf = [torch.tensor(f, device="cuda") for f in fields]
    if not tiled:
        return tp, tf, None, None
    til = G.Tiling(mp, order, (8, 8, 8))
    perm = til.sort(tp, tp.shape[0])
    from cabana_gb300 import core
    core.permute_by(perm, tp, *tf)
    return tp, tf, til, perm.cpu().numpy()


@pytest.mark.parametrize("form_name,precision,tiled", FORMS)
def test_reference_constants(oracle, form_name, precision, tiled):
    """tstInterpolation3d.hpp:38-251 through the GPU path."""
    gm = M.createUniformGlobalMesh((-1.2, 0.1, 1.1), (-0.3, 9.5, 2.3), 0.1)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, (True, True, True)), 1)
    lm = M.createLocalMesh(lg)
    (i0, i1), (j0, j1), (k0, k1) = lg.ownedSpace(M.CELL)
    pts = np.array([lm.coordinates(M.CELL, (i, j, k)) for k in range(k0, k1) for j in range(j0, j1)
                    for i in range(i0, i1)])
    n = pts.shape[0]
    mp = M.mesh_params(lg)
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    tp, _, til, _ = sorted_inputs(mp, 1, pts, [], tiled)
    own = lg.ownedSpace(M.NODE)
    sl = tuple(slice(a, b) for a, b in own)
    scalar_pt = torch.full((n,), 3.5, dtype=dt, device="cuda")
    vector_pt = torch.full((n, 3), 3.5, dtype=dt, device="cuda")
    tensor_pt = torch.full((n, 3, 3), 3.5, dtype=dt, device="cuda")
    halo = G.createHalo(G.NodeHaloPattern(), 1)
    sgrid = G.createArray("s", G.createArrayLayout(lg, 1, M.Node), dt)
    vgrid = G.createArray("v", G.createArrayLayout(lg, 3, M.Node), dt)
    cases = [(G.createScalarValueP2G(scalar_pt, -0.5), sgrid, -1.75), (G.createVectorValueP2G(vector_pt, -0.5), vgrid, -1.75),
             (G.createScalarGradientP2G(scalar_pt, -0.5), vgrid, 0.0),
             (G.createVectorDivergenceP2G(vector_pt, -0.5), sgrid, 0.0),
             (G.createTensorDivergenceP2G(tensor_pt, -0.5), vgrid, 0.0)]
    atol = 1e-12 if precision == G.PLAIN_FP64 else 2e-5
    for f, arr, expect in cases:
        G.ArrayOp.assign(arr, 0.0, G.Ghost)
        G.p2g(f, tp, n, G.Spline(1), halo, arr, precision=precision, tiling=til)
        got = arr.view()[sl].double().cpu().numpy()
        np.testing.assert_allclose(got, expect, atol=atol, rtol=1e-6)
    G.ArrayOp.assign(sgrid, 0.0, G.Ghost)
    G.ArrayOp.assign(vgrid, 0.0, G.Ghost)
    G.ArrayOp.assign(sgrid, 3.5, G.Own)
    G.ArrayOp.assign(vgrid, 3.5, G.Own)
    g2p_cases = [(G.createScalarValueG2P, (n,), sgrid, -1.75), (G.createVectorValueG2P, (n, 3), vgrid, -1.75),
                 (G.createScalarGradientG2P, (n, 3), sgrid, 0.0), (G.createVectorGradientG2P, (n, 3, 3), vgrid, 0.0),
                 (G.createVectorDivergenceG2P, (n,), vgrid, 0.0)]
    for mk, shape, arr, expect in g2p_cases:
        x = torch.zeros(shape, dtype=dt, device="cuda")
        G.g2p(arr, halo, tp, n, G.Spline(1), mk(x, -0.5), precision=precision, tiling=til)
        np.testing.assert_allclose(x.double().cpu().numpy(), expect, atol=atol, rtol=1e-6)


def _p2g_case(oracle, order, kind, precision, tiled, seed, clumped=False, n=3000, entity=M.NODE, dtype_grid=None):
    lg, mp = small_mesh(entity=entity)
    rng = np.random.default_rng(seed)
    lo, hi = domain(mp)
    pts = clumped_points(rng, n, lo, hi, 3, 0.5) if clumped else uniform_points(rng, n, lo, hi)
    x = rng.normal(size=(n, P2G_COMPS[kind]))
    om = oracle_mesh(oracle, mp)
    ref = np.zeros(mp.extents() + (P2G_DOFS[kind],))
    assert oracle.p2g(om, pts, order, [(kind, 0.75, x, ref)]) == 0
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    gdt = dtype_grid or dt
    tp, (tx,), til, _ = sorted_inputs(mp, order, pts, [x], tiled)
    shape = {1: (n,), 3: (n, 3), 9: (n, 3, 3)}[P2G_COMPS[kind]]
    tx = tx.to(dt).reshape(shape)
    arr = G.createArray("a", layout(lg, P2G_DOFS[kind], entity), gdt)
    mk = [G.createScalarValueP2G, G.createVectorValueP2G, G.createScalarGradientP2G, G.createVectorDivergenceP2G,
          G.createTensorDivergenceP2G][kind]
    G.p2g(mk(tx, 0.75), tp, n, G.Spline(order), G.createHalo(G.NodeHaloPattern(), mp.halo_width), arr,
          precision=precision, tiling=til, check_bounds=True)
    assert G.last_dispatch() == ("tiled" if tiled and order in (1, 2, 3) else "points")
    return arr.view().double().cpu().numpy(), ref


@pytest.mark.parametrize("form_name,precision,tiled", FORMS)
@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("kind", range(5))
def test_p2g_vs_oracle(oracle, form_name, precision, tiled, order, kind):
    if precision == G.FP32_COMPENSATED and order in (0, 4, 5, 6) and tiled:
        pytest.skip("tiled kernels cover orders 1-3")
    got, ref = _p2g_case(oracle, order, kind, precision, tiled, seed=100 * order + kind)
    tol = TOL_FP64 if precision == G.PLAIN_FP64 else (TOL_P2G_FP32 if tiled else TOL_P2G_FP32_POINTS)
    assert max_rel(got, ref) <= tol, (form_name, order, kind, max_rel(got, ref))


def _g2p_case(oracle, order, kind, precision, tiled, seed, n=3000, entity=M.NODE):
    lg, mp = small_mesh(entity=entity)
    rng = np.random.default_rng(seed)
    lo, hi = domain(mp)
    pts = uniform_points(rng, n, lo, hi)
    grid = rng.normal(size=mp.extents() + (G2P_DOFS[kind],))
    x0 = rng.normal(size=(n, G2P_COMPS[kind]))
    ref = x0.copy()
    om = oracle_mesh(oracle, mp)
    assert oracle.g2p(om, pts, order, [(kind, -1.25, ref, grid.copy())]) == 0
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    tp, (tx,), til, perm = sorted_inputs(mp, order, pts, [x0], tiled)
    shape = {1: (n,), 3: (n, 3), 9: (n, 3, 3)}[G2P_COMPS[kind]]
    tx = tx.to(dt).reshape(shape).contiguous()
    arr = G.createArray("a", layout(lg, G2P_DOFS[kind], entity), dt)
    arr.view().copy_(torch.tensor(grid, device="cuda").to(dt))
    mk = [G.createScalarValueG2P, G.createVectorValueG2P, G.createScalarGradientG2P, G.createVectorGradientG2P,
          G.createVectorDivergenceG2P][kind]
    G.g2p(arr, G.createHalo(G.NodeHaloPattern(), mp.halo_width), tp, n, G.Spline(order), mk(tx, -1.25),
          precision=precision, tiling=til, check_bounds=True)
    assert G.last_dispatch() == ("tiled" if tiled and order in (1, 2, 3) else "points")
    got = tx.double().cpu().numpy().reshape(n, -1)
    if perm is not None:
        ref = ref[perm]
        x0 = x0[perm]
    return got - x0, ref - x0


@pytest.mark.parametrize("form_name,precision,tiled", FORMS)
@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("kind", range(5))
def test_g2p_vs_oracle(oracle, form_name, precision, tiled, order, kind):
    if precision == G.FP32_COMPENSATED and order in (0, 4, 5, 6) and tiled:
        pytest.skip("tiled kernels cover orders 1-3")
    got, ref = _g2p_case(oracle, order, kind, precision, tiled, seed=7 + 100 * order + kind)
    tol = TOL_FP64 if precision == G.PLAIN_FP64 else TOL_G2P_FP32
    assert max_rel(got, ref) <= tol, (form_name, order, kind, max_rel(got, ref))


@pytest.mark.parametrize("form_name,precision,tiled", FORMS)
def test_clumped_p2g_and_cell_entity(oracle, form_name, precision, tiled):
    got, ref = _p2g_case(oracle, 2, 1, precision, tiled, seed=5, clumped=True, n=20000)
    tol = TOL_FP64 if precision == G.PLAIN_FP64 else (TOL_P2G_FP32 if tiled else TOL_P2G_FP32_POINTS)
    assert max_rel(got, ref) <= tol
    got, ref = _p2g_case(oracle, 3, 4, precision, tiled, seed=6, entity=M.CELL)
    assert max_rel(got, ref) <= tol
    got, ref = _g2p_case(oracle, 2, 3, precision, tiled, seed=8, entity=M.CELL)
    assert max_rel(got, ref) <= (TOL_FP64 if precision == G.PLAIN_FP64 else TOL_G2P_FP32)


def test_fp32_form_into_double_arrays(oracle):
    got, ref = _p2g_case(oracle, 2, 0, G.FP32_COMPENSATED, True, seed=9, dtype_grid=torch.float64)
    assert max_rel(got, ref) <= TOL_P2G_FP32


@pytest.mark.parametrize("form_name,precision,tiled", FORMS)
def test_fused_ops_match_oracle(oracle, form_name, precision, tiled):
    """The MPM transfer op set: mass + momentum + stress divergence, then
    velocity + velocity gradient, in one p2g and one g2p launch."""
    lg, mp = small_mesh()
    rng = np.random.default_rng(42)
    n = 8000
    lo, hi = domain(mp)
    pts = clumped_points(rng, n, lo, hi, 4, 0.6)
    m = rng.uniform(0.5, 1.5, size=(n, 1))
    v = rng.normal(size=(n, 3))
    mom = m * v
    sig = rng.normal(size=(n, 9))
    om = oracle_mesh(oracle, mp)
    mass_ref = np.zeros(mp.extents() + (1,))
    mom_ref = np.zeros(mp.extents() + (3,))
    frc_ref = np.zeros(mp.extents() + (3,))
    oracle.p2g(om, pts, 2, [(0, 1.0, m, mass_ref), (1, 1.0, mom, mom_ref), (4, -1.0, sig, frc_ref)])
    vel_ref = np.zeros((n, 3))
    vg_ref = np.zeros((n, 9))
    oracle.g2p(om, pts, 2, [(1, 1.0, vel_ref, mom_ref.copy()), (3, 1.0, vg_ref, mom_ref.copy())])

    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    tp, (tm, tmom, tsig), til, perm = sorted_inputs(mp, 2, pts, [m, mom, sig], tiled)
    tm, tmom, tsig = tm.to(dt).reshape(n), tmom.to(dt), tsig.to(dt).reshape(n, 3, 3)
    mass = G.createArray("mass", layout(lg, 1), dt)
    momg = G.createArray("mom", layout(lg, 3), dt)
    frc = G.createArray("frc", layout(lg, 3), dt)
    G.p2g([G.createScalarValueP2G(tm, 1.0), G.createVectorValueP2G(tmom, 1.0), G.createTensorDivergenceP2G(tsig, -1.0)],
          tp, n, G.Spline(2), None, [mass, momg, frc], precision=precision, tiling=til)
    vel = torch.zeros((n, 3), dtype=dt, device="cuda")
    vg = torch.zeros((n, 3, 3), dtype=dt, device="cuda")
    G.g2p(momg, None, tp, n, G.Spline(2), [G.createVectorValueG2P(vel, 1.0), G.createVectorGradientG2P(vg, 1.0)],
          precision=precision, tiling=til)
    tol_p = TOL_FP64 if precision == G.PLAIN_FP64 else (TOL_P2G_FP32 if tiled else TOL_P2G_FP32_POINTS)
    tol_g = TOL_FP64 if precision == G.PLAIN_FP64 else 4 * TOL_G2P_FP32
    assert max_rel(mass.view().double().cpu().numpy(), mass_ref) <= tol_p
    assert max_rel(momg.view().double().cpu().numpy(), mom_ref) <= tol_p
    assert max_rel(frc.view().double().cpu().numpy(), frc_ref) <= tol_p
    if perm is not None:
        vel_ref, vg_ref = vel_ref[perm], vg_ref[perm]
    # g2p reads the GPU momentum grid; compare against the oracle's g2p of the oracle grid
    assert max_rel(vel.double().cpu().numpy(), vel_ref) <= tol_g
    assert max_rel(vg.double().cpu().numpy().reshape(n, 9), vg_ref) <= tol_g
    # conservation of mass: grid total vs particle total
    assert abs(mass.view().double().sum().item() - m.sum()) <= 1e-6 * m.sum()


@pytest.mark.parametrize("offset", [0, 1, 2, 3])
def test_tiled_dense_fields_at_any_alignment(oracle, offset):
    """Dense FP32 point fields starting at any 4-byte offset inside a larger
    buffer: the tiled kernels stage them by bulk copies from the 16-byte
    boundary at or below the first element and write G2P results back by a
    bulk copy of the aligned interior plus plain stores of the ends. Values
    of the buffer outside the field are never written."""
    lg, mp = small_mesh()
    rng = np.random.default_rng(50 + offset)
    n = 5001
    lo, hi = domain(mp)
    pts = clumped_points(rng, n, lo, hi, 3, 0.6)
    v = rng.normal(size=(n, 3))
    x0 = rng.normal(size=(n, 9))
    om = oracle_mesh(oracle, mp)
    grid_ref = np.zeros(mp.extents() + (3,))
    assert oracle.p2g(om, pts, 2, [(1, 1.5, v, grid_ref)]) == 0
    tp, (tv, tx), til, perm = sorted_inputs(mp, 2, pts, [v, x0], True)

    def embed(t):
        flat = t.float().reshape(-1)
        buf = torch.full((flat.numel() + 8,), 7.0, device="cuda")
        buf[offset:offset + flat.numel()] = flat
        return buf, buf[offset:offset + flat.numel()].view(t.shape)

    _, tv32 = embed(tv)
    xbuf, tx32 = embed(tx.reshape(n, 3, 3))
    arr = G.createArray("a", layout(lg, 3), torch.float32)
    G.p2g(G.createVectorValueP2G(tv32, 1.5), tp, n, G.Spline(2), None, arr, precision=G.FP32_COMPENSATED, tiling=til)
    assert G.last_dispatch() == "tiled"
    assert max_rel(arr.view().double().cpu().numpy(), grid_ref) <= TOL_P2G_FP32

    grid = rng.normal(size=mp.extents() + (3,))
    ref = x0.copy()
    assert oracle.g2p(om, pts, 2, [(3, -0.5, ref, grid.copy())]) == 0
    garr = G.createArray("g", layout(lg, 3), torch.float32)
    garr.view().copy_(torch.tensor(grid, device="cuda").float())
    G.g2p(garr, None, tp, n, G.Spline(2), G.createVectorGradientG2P(tx32, -0.5), precision=G.FP32_COMPENSATED,
          tiling=til)
    assert G.last_dispatch() == "tiled"
    got = tx32.double().cpu().numpy().reshape(n, 9)
    ref, x0p = ref[perm], x0[perm]
    assert max_rel(got - x0p, ref - x0p) <= TOL_G2P_FP32
    guard = torch.cat([xbuf[:offset], xbuf[offset + 9 * n:]])
    assert bool(torch.all(guard == 7.0))


def test_aosoa_and_layout_left_fields(oracle):
    """Slice (AoSoA, VL=32) and LayoutLeft particle fields give the same result."""
    lg, mp = small_mesh()
    rng = np.random.default_rng(3)
    n = 1000
    lo, hi = domain(mp)
    pts = uniform_points(rng, n, lo, hi)
    v = rng.normal(size=(n, 3))
    ref = np.zeros(mp.extents() + (3,))
    oracle.p2g(oracle_mesh(oracle, mp), pts, 3, [(1, 2.0, v, ref)])
    # AoSoA<double[3] pos, double[3] vel>, VL = 32: SoA = pos[3][32] then vel[3][32]
    vl = 32
    nsoa = (n + vl - 1) // vl
    storage = torch.zeros(nsoa * 6 * vl, dtype=torch.float64, device="cuda")
    s = storage.view(nsoa, 2, 3, vl)
    pad = nsoa * vl - n
    s[:, 0] = torch.tensor(np.concatenate([pts, np.zeros((pad, 3))]).reshape(nsoa, vl, 3).transpose(0, 2, 1), device="cuda")
    s[:, 1] = torch.tensor(np.concatenate([v, np.zeros((pad, 3))]).reshape(nsoa, vl, 3).transpose(0, 2, 1), device="cuda")
    pos_slice = G.Slice(storage, 0, vl, 6 * vl, 3, n)
    vel_slice = G.Slice(storage, 3 * vl, vl, 6 * vl, 3, n)
    arr = G.createArray("a", layout(lg, 3))
    G.p2g(G.createVectorValueP2G(vel_slice, 2.0), pos_slice, n, G.Spline(3), None, arr)
    assert max_rel(arr.view().cpu().numpy(), ref) <= TOL_FP64
    # LayoutLeft: (3, n) storage viewed as (n, 3)
    left_pts = torch.tensor(pts.T.copy(), device="cuda").t()
    left_v = torch.tensor(v.T.copy(), device="cuda").t()
    arr2 = G.createArray("b", layout(lg, 3))
    G.p2g(G.createVectorValueP2G(left_v, 2.0), left_pts, n, G.Spline(3), None, arr2)
    assert max_rel(arr2.view().cpu().numpy(), ref) <= TOL_FP64


@pytest.mark.parametrize("precision", [G.PLAIN_FP64, G.FP32_COMPENSATED])
def test_periodic_halo_random(oracle, precision):
    lg, mp = small_mesh(periodic=(True, False, True), halo=2)
    rng = np.random.default_rng(12)
    n = 4000
    lo, hi = domain(mp)
    pts = uniform_points(rng, n, lo, hi)
    x = rng.normal(size=(n, 3))
    om = oracle_mesh(oracle, mp)
    ref = np.zeros(mp.extents() + (3,))
    oracle.p2g(om, pts, 2, [(1, 1.0, x, ref)])
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    arr = G.createArray("a", layout(lg, 3), dt)
    G.p2g(G.createVectorValueP2G(torch.tensor(x, device="cuda").to(dt), 1.0), torch.tensor(pts, device="cuda"), n,
          G.Spline(2), G.createHalo(G.NodeHaloPattern(), 2), arr, precision=precision)
    tol = TOL_FP64 if precision == G.PLAIN_FP64 else TOL_P2G_FP32
    assert max_rel(arr.view().double().cpu().numpy(), ref) <= tol
    # gather fills ghosts from owned images
    g = rng.normal(size=mp.extents() + (3,))
    gref = g.copy()
    oracle.halo_gather(om, gref)
    arr.view().copy_(torch.tensor(g, device="cuda").to(dt))
    G.createHalo(G.NodeHaloPattern(), 2).gather(arr)
    assert max_rel(arr.view().double().cpu().numpy(), gref) <= (0 if precision == G.PLAIN_FP64 else 1e-7)


@pytest.mark.parametrize("precision", [G.PLAIN_FP64, G.FP32_COMPENSATED])
def test_out_of_bounds_points_are_reported_and_skipped(oracle, precision):
    lg, mp = small_mesh(halo=1)
    rng = np.random.default_rng(1)
    n = 500
    lo, hi = domain(mp)
    pts = uniform_points(rng, n, lo, hi)
    pts[17] = (hi[0] + 5.0, lo[1], lo[2])   # far outside the ghosted space
    pts[18] = (lo[0] - 9.0, lo[1], lo[2])
    x = rng.normal(size=(n, 1))
    ref = np.zeros(mp.extents() + (1,))
    skipped = oracle.p2g(oracle_mesh(oracle, mp), pts, 3, [(0, 1.0, x, ref)])
    assert skipped == 2
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    arr = G.createArray("a", layout(lg, 1), dt)
    with pytest.raises(Exception) as e:
        G.p2g(G.createScalarValueP2G(torch.tensor(x[:, 0], device="cuda").to(dt), 1.0), torch.tensor(pts, device="cuda"),
              n, G.Spline(3), None, arr, precision=precision, check_bounds=True)
    assert "ghosted" in str(e.value)
    tol = TOL_FP64 if precision == G.PLAIN_FP64 else TOL_P2G_FP32
    assert max_rel(arr.view().double().cpu().numpy(), ref) <= tol


def test_empty_point_set():
    lg, mp = small_mesh()
    arr = G.createArray("a", layout(lg, 1))
    x = torch.zeros(0, dtype=torch.float64, device="cuda")
    pts = torch.zeros((0, 3), dtype=torch.float64, device="cuda")
    G.p2g(G.createScalarValueP2G(x, 1.0), pts, 0, G.Spline(2), None, arr)
    G.g2p(arr, None, pts, 0, G.Spline(2), G.createScalarValueG2P(x, 1.0))
    assert arr.view().abs().sum().item() == 0.0


@pytest.mark.parametrize("layout_name", ["layout_left", "aosoa"])
def test_tiled_fp32_with_strided_and_aosoa_fields(oracle, layout_name):
    """The tiled FP32 kernels on point fields that are not dense rows: a
    LayoutLeft View (components n apart) or AoSoA slices (VL = 32), staged
    component by component. Mass + momentum + stress divergence, then
    velocity + velocity gradient."""
    lg, mp = small_mesh()
    rng = np.random.default_rng(77)
    n = 6000
    lo, hi = domain(mp)
    pts = clumped_points(rng, n, lo, hi, 4, 0.6)
    m = rng.uniform(0.5, 1.5, size=(n, 1))
    mom = m * rng.normal(size=(n, 3))
    sig = rng.normal(size=(n, 9))
    om = oracle_mesh(oracle, mp)
    mass_ref = np.zeros(mp.extents() + (1,))
    mom_ref = np.zeros(mp.extents() + (3,))
    frc_ref = np.zeros(mp.extents() + (3,))
    oracle.p2g(om, pts, 2, [(0, 1.0, m, mass_ref), (1, 1.0, mom, mom_ref), (4, -1.0, sig, frc_ref)])
    vel_ref = np.zeros((n, 3))
    vg_ref = np.zeros((n, 9))
    oracle.g2p(om, pts, 2, [(1, 1.0, vel_ref, mom_ref.copy()), (3, 1.0, vg_ref, mom_ref.copy())])
    # tile order, applied on the host so every layout holds sorted data
    til = G.Tiling(mp, 2, (8, 8, 8))
    perm = til.sort(torch.tensor(pts, device="cuda"), n).cpu().numpy()
    pts_s, m_s, mom_s, sig_s = pts[perm], m[perm], mom[perm], sig[perm]
    tp = torch.tensor(pts_s, device="cuda")
    f32 = torch.float32
    if layout_name == "layout_left":
        tm = torch.tensor(m_s[:, 0], device="cuda").to(f32)
        tmom = torch.tensor(mom_s.T.copy(), device="cuda").to(f32).t()                     # (n, 3), strides (1, n)
        tsig = torch.tensor(sig_s.reshape(n, 3, 3).transpose(1, 2, 0).copy(), device="cuda").to(f32).permute(2, 0, 1)
        vel = torch.zeros((3, n), dtype=f32, device="cuda").t()
        vg = torch.zeros((3, 3, n), dtype=f32, device="cuda").permute(2, 0, 1)
        read_vel = lambda: vel.double().cpu().numpy()  # noqa: E731
        read_vg = lambda: vg.double().cpu().numpy().reshape(n, 9)  # noqa: E731
    else:
        vl = 32
        nsoa = (n + vl - 1) // vl
        pad = nsoa * vl - n

        def soa(a):  # (n, c) -> (nsoa, c, vl)
            return np.concatenate([a, np.zeros((pad, a.shape[1]))]).reshape(nsoa, vl, a.shape[1]).transpose(0, 2, 1)

        # AoSoA<float mass, float[3] mom, float[3][3] stress>: 13 floats x VL per SoA
        storage = torch.tensor(np.concatenate([soa(m_s), soa(mom_s), soa(sig_s)], axis=1).reshape(-1), device="cuda").to(f32)
        tm = G.Slice(storage, 0, vl, 13 * vl, 1, n)
        tmom = G.Slice(storage, vl, vl, 13 * vl, 3, n)
        tsig = G.Slice(storage, 4 * vl, vl, 13 * vl, 9, n)
        # AoSoA<float[3] vel, float[3][3] velgrad>: 12 floats x VL per SoA
        out = torch.zeros(nsoa * 12 * vl, dtype=f32, device="cuda")
        vel = G.Slice(out, 0, vl, 12 * vl, 3, n)
        vg = G.Slice(out, 3 * vl, vl, 12 * vl, 9, n)

        def unsoa(first, c):
            a = out.double().cpu().numpy().reshape(nsoa, 12, vl)[:, first:first + c, :]
            return a.transpose(0, 2, 1).reshape(nsoa * vl, c)[:n]

        read_vel = lambda: unsoa(0, 3)  # noqa: E731
        read_vg = lambda: unsoa(3, 9)  # noqa: E731
    mass = G.createArray("mass", layout(lg, 1), f32)
    momg = G.createArray("mom", layout(lg, 3), f32)
    frc = G.createArray("frc", layout(lg, 3), f32)
    G.p2g([G.createScalarValueP2G(tm, 1.0), G.createVectorValueP2G(tmom, 1.0), G.createTensorDivergenceP2G(tsig, -1.0)],
          tp, n, G.Spline(2), None, [mass, momg, frc], precision=G.FP32_COMPENSATED, tiling=til, check_bounds=True)
    assert G.last_dispatch() == "tiled"
    for got, ref in [(mass, mass_ref), (momg, mom_ref), (frc, frc_ref)]:
        assert max_rel(got.view().double().cpu().numpy(), ref) <= TOL_P2G_FP32, layout_name
    G.g2p(momg, None, tp, n, G.Spline(2), [G.createVectorValueG2P(vel, 1.0), G.createVectorGradientG2P(vg, 1.0)],
          precision=G.FP32_COMPENSATED, tiling=til, check_bounds=True)
    assert G.last_dispatch() == "tiled"
    assert max_rel(read_vel(), vel_ref[perm]) <= 4 * TOL_G2P_FP32, layout_name
    assert max_rel(read_vg(), vg_ref[perm]) <= 4 * TOL_G2P_FP32, layout_name
