"""GPU parity of 2D p2g / g2p against the FP64 oracle, through the C ABI.

The 2D specialisations of grid/src/Cabana_Grid_Interpolation.hpp run on the
point kernels (one thread per point) in both precision forms. Tolerances
(max|gpu - oracle| / max|oracle|):
  * CGX_PLAIN_FP64:        1e-12 (atomic summation order only)
  * CGX_FP32_COMPENSATED:  P2G grid 4e-6 (plain float atomics), G2P 2e-6
"""
import numpy as np
import pytest
import torch

from cabana_gb300 import grid as G
from cabana_gb300 import mesh as M
from tests.helpers import max_rel

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_P2G_FP32 = 4e-6
TOL_G2P_FP32 = 2e-6

P2G_COMPS_2D = {0: 1, 1: 2, 2: 1, 3: 2, 4: 4}
P2G_DOFS_2D = {0: 1, 1: 2, 2: 2, 3: 1, 4: 2}
G2P_COMPS_2D = {0: 1, 1: 2, 2: 2, 3: 4, 4: 1}
G2P_DOFS_2D = {0: 1, 1: 2, 2: 1, 3: 2, 4: 2}
P2G_MAKERS = [G.createScalarValueP2G, G.createVectorValueP2G, G.createScalarGradientP2G, G.createVectorDivergenceP2G,
              G.createTensorDivergenceP2G]
G2P_MAKERS = [G.createScalarValueG2P, G.createVectorValueG2P, G.createScalarGradientG2P, G.createVectorGradientG2P,
              G.createVectorDivergenceG2P]
SHAPES = {1: lambda n: (n,), 2: lambda n: (n, 2), 4: lambda n: (n, 2, 2)}
FORMS = [("plain64", G.PLAIN_FP64), ("fp32", G.FP32_COMPENSATED)]


def mesh2d(periodic=(False, False), halo=3, entity=M.NODE):
    gm = M.createUniformGlobalMesh((-1.3, 2.1), (-1.3 + 14 * 0.37, 2.1 + 11 * 0.37), 0.37)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, periodic), halo)
    return lg, M.mesh_params(lg, entity)


def oracle_mesh2(oracle, mp):
    return oracle.make_mesh(mp.ghost_low, mp.cell_size, mp.owned_cells, mp.halo_width, mp.periodic, mp.entity,
                            num_space_dim=2)


def owned_box(mp):
    lo = tuple(mp.ghost_low[d] + mp.halo_width * mp.cell_size[d] for d in range(2))
    hi = tuple(lo[d] + mp.owned_cells[d] * mp.cell_size[d] for d in range(2))
    return lo, hi


def points2d(rng, n, mp):
    lo, hi = owned_box(mp)
    return np.stack([rng.uniform(lo[d], hi[d], n) for d in range(2)], axis=1)


@pytest.mark.parametrize("form_name,precision", FORMS)
def test_reference_constants_2d(form_name, precision):
    """tstInterpolation2d.hpp through the GPU path."""
    gm = M.createUniformGlobalMesh((-1.2, 0.1), (-0.2, 9.5), 0.1)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, (True, True)), 1)
    lm = M.createLocalMesh(lg)
    (i0, i1), (j0, j1) = lg.ownedSpace(M.CELL)
    pts = np.array([lm.coordinates(M.CELL, (i, j)) for j in range(j0, j1) for i in range(i0, i1)])
    n = pts.shape[0]
    tp = torch.tensor(pts, device="cuda")
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    own = tuple(slice(a, b) for a, b in lg.ownedSpace(M.NODE))
    halo = G.createHalo(G.NodeHaloPattern(), 1)
    sgrid = G.createArray("s", G.createArrayLayout(lg, 1, M.Node), dt)
    vgrid = G.createArray("v", G.createArrayLayout(lg, 2, M.Node), dt)
    assert tuple(sgrid.view().shape) == (13, 97, 1)
    atol = 1e-12 if precision == G.PLAIN_FP64 else 2e-5
    for kind, arr, expect in [(0, sgrid, -1.75), (1, vgrid, -1.75), (2, vgrid, 0.0), (3, sgrid, 0.0), (4, vgrid, 0.0)]:
        x = torch.full(SHAPES[P2G_COMPS_2D[kind]](n), 3.5, dtype=dt, device="cuda")
        G.ArrayOp.assign(arr, 0.0, G.Ghost)
        G.p2g(P2G_MAKERS[kind](x, -0.5), tp, n, G.Spline(1), halo, arr, precision=precision)
        assert G.last_dispatch() == "points"
        np.testing.assert_allclose(arr.view()[own].double().cpu().numpy(), expect, atol=atol, rtol=1e-6)
    G.ArrayOp.assign(sgrid, 0.0, G.Ghost)
    G.ArrayOp.assign(vgrid, 0.0, G.Ghost)
    G.ArrayOp.assign(sgrid, 3.5, G.Own)
    G.ArrayOp.assign(vgrid, 3.5, G.Own)
    for kind, arr, expect in [(0, sgrid, -1.75), (1, vgrid, -1.75), (2, sgrid, 0.0), (3, vgrid, 0.0), (4, vgrid, 0.0)]:
        x = torch.zeros(SHAPES[G2P_COMPS_2D[kind]](n), dtype=dt, device="cuda")
        G.g2p(arr, halo, tp, n, G.Spline(1), G2P_MAKERS[kind](x, -0.5), precision=precision)
        np.testing.assert_allclose(x.double().cpu().numpy(), expect, atol=atol, rtol=1e-6)


@pytest.mark.parametrize("form_name,precision", FORMS)
@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("kind", range(5))
def test_p2g_vs_oracle_2d(oracle, form_name, precision, order, kind):
    lg, mp = mesh2d()
    rng = np.random.default_rng(500 + 10 * order + kind)
    n = 2500
    pts = points2d(rng, n, mp)
    x = rng.normal(size=(n, P2G_COMPS_2D[kind]))
    ref = np.zeros(mp.extents() + (P2G_DOFS_2D[kind],))
    assert oracle.p2g(oracle_mesh2(oracle, mp), pts, order, [(kind, 0.75, x, ref)]) == 0
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    tx = torch.tensor(x, device="cuda").to(dt).reshape(SHAPES[P2G_COMPS_2D[kind]](n))
    arr = G.createArray("a", G.createArrayLayout(lg, P2G_DOFS_2D[kind], M.Node), dt)
    G.p2g(P2G_MAKERS[kind](tx, 0.75), torch.tensor(pts, device="cuda"), n, G.Spline(order),
          G.createHalo(G.NodeHaloPattern(), mp.halo_width), arr, precision=precision, check_bounds=True)
    tol = TOL_FP64 if precision == G.PLAIN_FP64 else TOL_P2G_FP32
    assert max_rel(arr.view().double().cpu().numpy(), ref) <= tol, (form_name, order, kind)


@pytest.mark.parametrize("form_name,precision", FORMS)
@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("kind", range(5))
def test_g2p_vs_oracle_2d(oracle, form_name, precision, order, kind):
    lg, mp = mesh2d(entity=M.CELL if kind == 3 else M.NODE)
    rng = np.random.default_rng(700 + 10 * order + kind)
    n = 2500
    pts = points2d(rng, n, mp)
    grid = rng.normal(size=mp.extents() + (G2P_DOFS_2D[kind],))
    x0 = rng.normal(size=(n, G2P_COMPS_2D[kind]))
    ref = x0.copy()
    assert oracle.g2p(oracle_mesh2(oracle, mp), pts, order, [(kind, -1.25, ref, grid.copy())]) == 0
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    tx = torch.tensor(x0, device="cuda").to(dt).reshape(SHAPES[G2P_COMPS_2D[kind]](n)).contiguous()
    ent = M.Cell if kind == 3 else M.Node
    arr = G.createArray("a", G.createArrayLayout(lg, G2P_DOFS_2D[kind], ent), dt)
    arr.view().copy_(torch.tensor(grid, device="cuda").to(dt))
    G.g2p(arr, G.createHalo(G.NodeHaloPattern(), mp.halo_width), torch.tensor(pts, device="cuda"), n, G.Spline(order),
          G2P_MAKERS[kind](tx, -1.25), precision=precision, check_bounds=True)
    got = tx.double().cpu().numpy().reshape(n, -1)
    tol = TOL_FP64 if precision == G.PLAIN_FP64 else TOL_G2P_FP32
    assert max_rel(got - x0, ref - x0) <= tol, (form_name, order, kind)


@pytest.mark.parametrize("form_name,precision", FORMS)
def test_periodic_halo_and_fused_ops_2d(oracle, form_name, precision):
    """Periodic in i only; mass + momentum + stress divergence in one p2g,
    velocity + velocity gradient in one g2p; conservation of mass."""
    lg, mp = mesh2d(periodic=(True, False), halo=2)
    rng = np.random.default_rng(31)
    n = 6000
    pts = points2d(rng, n, mp)
    lo, hi = owned_box(mp)
    pts[:, 1] = rng.uniform(lo[1] + 3 * 0.37, hi[1] - 3 * 0.37, n)  # stencils stay in owned j rows
    m = rng.uniform(0.5, 1.5, size=(n, 1))
    mom = rng.normal(size=(n, 2))
    sig = rng.normal(size=(n, 4))
    om = oracle_mesh2(oracle, mp)
    mass_ref = np.zeros(mp.extents() + (1,))
    mom_ref = np.zeros(mp.extents() + (2,))
    frc_ref = np.zeros(mp.extents() + (2,))
    oracle.p2g(om, pts, 2, [(0, 1.0, m, mass_ref), (1, 1.0, mom, mom_ref), (4, -1.0, sig, frc_ref)])
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    tp = torch.tensor(pts, device="cuda")
    tm = torch.tensor(m[:, 0], device="cuda").to(dt)
    tmom = torch.tensor(mom, device="cuda").to(dt)
    tsig = torch.tensor(sig, device="cuda").to(dt).reshape(n, 2, 2)
    mass = G.createArray("mass", G.createArrayLayout(lg, 1, M.Node), dt)
    momg = G.createArray("mom", G.createArrayLayout(lg, 2, M.Node), dt)
    frc = G.createArray("frc", G.createArrayLayout(lg, 2, M.Node), dt)
    halo = G.createHalo(G.NodeHaloPattern(), 2)
    G.p2g([G.createScalarValueP2G(tm, 1.0), G.createVectorValueP2G(tmom, 1.0), G.createTensorDivergenceP2G(tsig, -1.0)],
          tp, n, G.Spline(2), halo, [mass, momg, frc], precision=precision)
    tol = TOL_FP64 if precision == G.PLAIN_FP64 else TOL_P2G_FP32
    for got, ref in [(mass, mass_ref), (momg, mom_ref), (frc, frc_ref)]:
        assert max_rel(got.view().double().cpu().numpy(), ref) <= tol
    own = tuple(slice(a, b) for a, b in lg.ownedSpace(M.NODE))
    assert abs(mass.view()[own].double().sum().item() - m.sum()) <= 1e-5 * m.sum()
    vel_ref = np.zeros((n, 2))
    vg_ref = np.zeros((n, 4))
    oracle.g2p(om, pts, 2, [(1, 1.0, vel_ref, mom_ref.copy()), (3, 1.0, vg_ref, mom_ref.copy())])
    vel = torch.zeros((n, 2), dtype=dt, device="cuda")
    vg = torch.zeros((n, 2, 2), dtype=dt, device="cuda")
    G.g2p(momg, halo, tp, n, G.Spline(2), [G.createVectorValueG2P(vel, 1.0), G.createVectorGradientG2P(vg, 1.0)],
          precision=precision)
    tol_g = TOL_FP64 if precision == G.PLAIN_FP64 else 4 * TOL_G2P_FP32
    assert max_rel(vel.double().cpu().numpy(), vel_ref) <= tol_g
    assert max_rel(vg.double().cpu().numpy().reshape(n, 4), vg_ref) <= tol_g


def test_out_of_bounds_points_are_reported_2d():
    lg, mp = mesh2d(halo=1)
    n = 100
    pts = np.zeros((n, 2))
    pts[:, 0] = mp.ghost_low[0] - 5.0  # every stencil leaves the ghosted space
    pts[:, 1] = mp.ghost_low[1] + 3.0
    arr = G.createArray("a", G.createArrayLayout(lg, 1, M.Node))
    x = torch.ones(n, dtype=torch.float64, device="cuda")
    with pytest.raises(Exception) as e:
        G.p2g(G.createScalarValueP2G(x, 1.0), torch.tensor(pts, device="cuda"), n, G.Spline(2), None, arr,
              check_bounds=True)
    assert "ghosted" in str(e.value)
    assert float(arr.view().abs().sum()) == 0.0
