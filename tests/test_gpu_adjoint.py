"""Adjoint parity on the GPU (cgx_p2g_adjoint / cgx_g2p_adjoint).

* Every forward kind (the reference's ten functors plus the two transposed
  tensor forms), orders 1-3, plain FP64 and FP32 forms, periodic and not:
  point-field, grid and position cotangents against the oracle adjoint
  (itself pinned by finite differences in tests/test_oracle_adjoint.py).
* The transpose identity on the GPU: <P2G(x), g> = <x, P2G^T g>.
* The adjoint workload on the 128^3 mesh with 2^24 uniform particles,
  Spline<3>, FP32: dL/dv against the oracle's g2p of the weights (the
  transpose) and dL/dx against an FP64 central difference (h = 1e-3) on
  1,024 sampled particles, tolerance 1e-5.
* torch.autograd.gradcheck of the test-only autograd Functions (FP64).

Tolerances: FP64 1e-11 (summation order); FP32 2e-5 of the largest entry.
"""
import numpy as np
import pytest
import torch

from cabana_gb300 import grid as G
from cabana_gb300 import mesh as M
from tests.helpers import G2P_COMPS, G2P_DOFS, P2G_COMPS, P2G_DOFS, clumped_points, domain, max_rel, oracle_mesh

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-11
TOL_FP32 = 2e-5

P2G_FACTORY = [G.createScalarValueP2G, G.createVectorValueP2G, G.createScalarGradientP2G,
               G.createVectorDivergenceP2G, G.createTensorDivergenceP2G, G.createTensorDivergenceTransposedP2G]
G2P_FACTORY = [G.createScalarValueG2P, G.createVectorValueG2P, G.createScalarGradientG2P,
               G.createVectorGradientG2P, G.createVectorDivergenceG2P, G.createVectorGradientTransposedG2P]
SHAPE = {1: lambda n: (n,), 3: lambda n: (n, 3), 9: lambda n: (n, 3, 3)}


def _case(oracle, periodic, seed, n=3000):
    lg, mp = M.simple_mesh(10, 0.37, (-1.1, 0.4, 2.0), 2, periodic=(periodic,) * 3)
    lo, hi = domain(mp)
    rng = np.random.default_rng(seed)
    pts = clumped_points(rng, n, lo, hi, 3, 0.6)
    return lg, mp, oracle_mesh(oracle, mp), pts, rng


def _forms(order):
    yield G.PLAIN_FP64, torch.float64, None
    yield G.FP32_COMPENSATED, torch.float32, None
    yield G.FP32_COMPENSATED, torch.float32, "tiled"


def _sorted(lg, mp, order, pts, arrays_np):
    """Tile-sort the points (and per-point numpy arrays) for the tiled path."""
    dev = torch.device("cuda")
    pos = torch.tensor(pts, dtype=torch.float64, device=dev)
    til = G.Tiling(mp, order, (8, 8, 8), device=dev)
    perm = til.sort(pos, pos.shape[0]).cpu().numpy()
    return til, pts[perm], [a[perm] for a in arrays_np]


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("kind", range(6))
def test_p2g_adjoint_matches_oracle(oracle, kind, order, periodic):
    lg, mp, om, pts0, rng = _case(oracle, periodic, 10 * kind + order)
    n = pts0.shape[0]
    x0 = rng.normal(size=(n, P2G_COMPS[kind]))
    gbar0 = rng.normal(size=mp.extents() + (P2G_DOFS[kind],))
    for precision, dt, mode in _forms(order):
        til, pts, (x,) = (None, pts0, (x0,)) if mode is None else _sorted(lg, mp, order, pts0, [x0])
        ref_xbar = np.zeros_like(x)
        ref_pbar = np.zeros_like(pts)
        oracle.p2g_adjoint(om, pts, order, [dict(kind=kind, mult=-0.6, x=x, x_bar=ref_xbar, array_bar=gbar0.copy())],
                           points_bar=ref_pbar)
        pos = torch.tensor(pts, device="cuda")
        xt = torch.tensor(x.reshape(SHAPE[P2G_COMPS[kind]](n)), dtype=dt, device="cuda")
        gbar = G.createArray("g", G.createArrayLayout(lg, P2G_DOFS[kind], G.Node), dt)
        gbar.view().copy_(torch.tensor(gbar0))
        xbar = torch.zeros_like(xt)
        pbar = torch.zeros_like(pos)
        G.p2g_adjoint(P2G_FACTORY[kind](xt, -0.6), pos, n, G.Spline(order), G.createHalo(G.NodeHaloPattern(), 1),
                      gbar, x_bar=xbar, points_bar=pbar, precision=precision, tiling=til)
        if mode == "tiled":
            assert G.last_dispatch() == "tiled"
        tol = TOL_FP64 if dt == torch.float64 else TOL_FP32
        assert max_rel(xbar.cpu().numpy().reshape(n, -1), ref_xbar) <= tol, (precision, mode)
        if np.abs(ref_pbar).max() > 0:
            assert max_rel(pbar.cpu().numpy(), ref_pbar) <= tol, (precision, mode)
        else:
            assert np.abs(pbar.cpu().numpy()).max() == 0.0


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("kind", range(6))
def test_g2p_adjoint_matches_oracle(oracle, kind, order, periodic):
    lg, mp, om, pts0, rng = _case(oracle, periodic, 20 * kind + order)
    n = pts0.shape[0]
    xbar0 = rng.normal(size=(n, G2P_COMPS[kind]))
    grid0 = rng.normal(size=mp.extents() + (G2P_DOFS[kind],))
    oracle.halo_gather(om, grid0)  # the array as the forward g2p read it
    for precision, dt, mode in _forms(order):
        til, pts, (xbar_np,) = (None, pts0, (xbar0,)) if mode is None else _sorted(lg, mp, order, pts0, [xbar0])
        ref_gbar = np.zeros_like(grid0)
        ref_pbar = np.zeros_like(pts)
        oracle.g2p_adjoint(om, pts, order, [dict(kind=kind, mult=0.8, x_bar=xbar_np, array=grid0, array_bar=ref_gbar)],
                           points_bar=ref_pbar)
        pos = torch.tensor(pts, device="cuda")
        xbar = torch.tensor(xbar_np.reshape(SHAPE[G2P_COMPS[kind]](n)), dtype=dt, device="cuda")
        arr = G.createArray("a", G.createArrayLayout(lg, G2P_DOFS[kind], G.Node), dt)
        arr.view().copy_(torch.tensor(grid0))
        gbar = G.createArray("g", G.createArrayLayout(lg, G2P_DOFS[kind], G.Node), dt)
        pbar = torch.zeros_like(pos)
        out = torch.zeros_like(xbar)
        G.g2p_adjoint(arr, G.createHalo(G.NodeHaloPattern(), 1), pos, n, G.Spline(order), G2P_FACTORY[kind](out, 0.8),
                      xbar, array_bar=gbar, points_bar=pbar, precision=precision, tiling=til)
        if mode == "tiled":
            assert G.last_dispatch() == "tiled"
        tol = TOL_FP64 if dt == torch.float64 else TOL_FP32
        assert max_rel(gbar.view().cpu().numpy(), ref_gbar) <= tol, (precision, mode)
        if np.abs(ref_pbar).max() > 0:
            assert max_rel(pbar.cpu().numpy(), ref_pbar) <= tol, (precision, mode)
        else:
            assert np.abs(pbar.cpu().numpy()).max() == 0.0


@pytest.mark.parametrize("kind", range(6))
def test_transpose_identity(kind):
    """<P2G(x), g> = <x, P2G^T g> for the plain FP64 form on a clumped set."""
    lg, mp = M.simple_mesh(12, 0.5, (0.0, 0.0, 0.0), 2)
    lo, hi = domain(mp)
    rng = np.random.default_rng(kind)
    n = 20000
    pos = torch.tensor(clumped_points(rng, n, lo, hi, 4, 0.8), device="cuda")
    x = torch.tensor(rng.normal(size=(n, P2G_COMPS[kind])).reshape(SHAPE[P2G_COMPS[kind]](n)), device="cuda")
    arr = G.createArray("a", G.createArrayLayout(lg, P2G_DOFS[kind], G.Node), torch.float64)
    G.p2g(P2G_FACTORY[kind](x, 1.5), pos, n, G.Spline(3), None, arr)
    g = G.createArray("g", G.createArrayLayout(lg, P2G_DOFS[kind], G.Node), torch.float64)
    g.view().copy_(torch.tensor(rng.normal(size=tuple(g.view().shape))))
    xbar = torch.zeros_like(x)
    G.p2g_adjoint(P2G_FACTORY[kind](x, 1.5), pos, n, G.Spline(3), None, g, x_bar=xbar)
    lhs = float((arr.view() * g.view()).sum())
    rhs = float((x * xbar).sum())
    assert abs(lhs - rhs) <= 1e-12 * (arr.view().abs() * g.view().abs()).sum().item()


def test_adjoint_workload_finite_differences(oracle):
    """128^3 cells, 2^24 uniform particles, Spline<3>, FP32 with an FP64 check.
    L = sum_nodes w . P2G(momentum), momentum = m v, w ~ N(0, 1) per node dof.
    dL/dv_p = m_p G2P(w)(x_p); dL/dx_p = sum_c mom_p[c] grad(G2P(w_c))(x_p)."""
    cells, n, order = 128, 1 << 24, 3
    lg, mp = M.simple_mesh(cells, 1.0, (0.0, 0.0, 0.0), 2)
    lo, hi = domain(mp)
    gen = torch.Generator(device="cuda").manual_seed(4)
    pos = torch.rand(n, 3, device="cuda", dtype=torch.float64, generator=gen) * cells
    mass = 0.5 + torch.rand(n, device="cuda", dtype=torch.float64, generator=gen)
    vel = torch.randn(n, 3, device="cuda", dtype=torch.float64, generator=gen)
    mom32 = (mass[:, None] * vel).float()
    w = G.createArray("w", G.createArrayLayout(lg, 3, G.Node), torch.float32)
    w.view().copy_(torch.randn(tuple(w.view().shape), device="cuda", generator=gen))
    til = G.Tiling(mp, order, (8, 8, 8), device="cuda")
    perm = til.sort(pos, n)
    pos, mass, vel, mom32 = pos[perm].contiguous(), mass[perm].contiguous(), vel[perm].contiguous(), mom32[perm].contiguous()
    mom_bar = torch.zeros_like(mom32)
    pos_bar = torch.zeros_like(pos)
    G.p2g_adjoint(G.createVectorValueP2G(mom32, 1.0), pos, n, G.Spline(order), None, w, x_bar=mom_bar,
                  points_bar=pos_bar, precision=G.FP32_COMPENSATED, tiling=til)
    assert G.last_dispatch() == "tiled"
    v_bar = mass[:, None] * mom_bar.double()
    # dL/dv on 1,024 sampled particles against the oracle's g2p of w (the transpose)
    idx = torch.randperm(n, device="cuda", generator=gen)[:1024]
    pts_s = pos[idx].cpu().numpy()
    om = oracle_mesh(oracle, mp)
    wg = w.view().double().cpu().numpy()
    ref = np.zeros((1024, 3))
    oracle.g2p(om, pts_s, order, [(1, 1.0, ref, wg.copy())])
    ref_vbar = mass[idx].cpu().numpy()[:, None] * ref
    assert max_rel(v_bar[idx].cpu().numpy(), ref_vbar) <= 1e-5
    # dL/dx: FP64 central difference, h = 1e-3, through the plain FP64 g2p of w
    h = 1e-3
    w64 = G.createArray("w64", G.createArrayLayout(lg, 3, G.Node), torch.float64)
    w64.view().copy_(w.view().double())
    mom_s = mom32[idx].double()  # the FP32 momentum the adjoint saw
    fd = torch.zeros(1024, 3, dtype=torch.float64, device="cuda")
    for e in range(3):
        vals = []
        for sgn in (1.0, -1.0):
            q = pos[idx].clone()
            q[:, e] += sgn * h
            out = torch.zeros(1024, 3, dtype=torch.float64, device="cuda")
            G.g2p(w64, None, q, 1024, G.Spline(order), G.createVectorValueG2P(out, 1.0))
            vals.append((out * mom_s).sum(dim=1))
        fd[:, e] = (vals[0] - vals[1]) / (2 * h)
    err = float((pos_bar[idx] - fd).abs().max() / fd.abs().max())
    assert err <= 1e-5, err


def test_autograd_functions_gradcheck():
    from tests.autograd_cgx import G2PVelocity, P2GMomentum, _Ctx
    lg, mp = M.simple_mesh(4, 0.5, (0.2, 0.0, -0.3), 2)
    lo, hi = domain(mp)
    rng = np.random.default_rng(7)
    n = 6
    ctx = _Ctx(lg, 3, G.PLAIN_FP64)
    pos = torch.tensor(rng.uniform(lo, hi, size=(n, 3)), device="cuda", requires_grad=True)
    mom = torch.tensor(rng.normal(size=(n, 3)), device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda p, m: P2GMomentum.apply(p, m, ctx, -0.5), (pos, mom), eps=1e-6, atol=1e-7,
                                    rtol=1e-5, nondet_tol=1e-12)
    grid = torch.tensor(rng.normal(size=mp.extents() + (3,)), device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda p, g: G2PVelocity.apply(p, g, ctx, 1.25), (pos, grid), eps=1e-6, atol=1e-7,
                                    rtol=1e-5, nondet_tol=1e-12)

    # the composed transfer: positions enter both directions
    def chain(p, m):
        g = P2GMomentum.apply(p, m, ctx, 1.0)
        return G2PVelocity.apply(p, g, ctx, 1.0)
    # atomics in the grid adjoint make repeated backward passes differ in the last bits
    assert torch.autograd.gradcheck(chain, (pos, mom), eps=1e-6, atol=1e-7, rtol=1e-5, nondet_tol=1e-12)
