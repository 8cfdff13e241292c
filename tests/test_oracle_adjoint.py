"""Pins the oracle's adjoint restatement (no reference counterpart).

* Spline second derivatives: agree with a central difference of the
  reference gradient formulas, sum to zero (derivative of the partition of
  unity, tstSplines.cpp:25-518 style), annihilate linear node coordinates and
  give 2 r^2 on squared node coordinates for orders >= 2 (quadratic
  reproduction).
* p2g / g2p adjoints: the position derivative agrees with a central
  difference of the oracle forward in FP64, and the point-field / grid
  derivative satisfies the dot-product identity <dL/dy, dy> = dL for random
  directions dy (the forward operators are linear in y).
"""
import numpy as np
import pytest

from cabana_gb300 import mesh as M
from tests.helpers import G2P_COMPS, G2P_DOFS, P2G_COMPS, P2G_DOFS, domain, oracle_mesh


@pytest.mark.parametrize("order", range(7))
def test_hessian_known_answers(oracle, order):
    rng = np.random.default_rng(order)
    r = 1.7
    for x0 in rng.uniform(2.0, 9.0, size=12):
        h = oracle.spline_hessian(order, x0, r)
        step = 1e-6
        fd = (oracle.spline_gradient(order, x0 + step, r) - oracle.spline_gradient(order, x0 - step, r)) / (2 * step) * r
        assert np.allclose(h, fd, rtol=0, atol=1e-8 * r * r)
        assert abs(h.sum()) < 1e-13 * r * r
        s = oracle.spline_stencil(order, x0).astype(np.float64)
        assert abs((h * s).sum()) < 1e-11 * r * r
        if order >= 2:
            assert abs((h * s * s).sum() - 2.0 * r * r) < 1e-9 * r * r


def _setup(oracle, order, periodic, seed, n=8):
    lg, mp = M.simple_mesh(6, 0.5, (0.3, -0.2, 0.1), 2, periodic=(periodic,) * 3)
    om = oracle_mesh(oracle, mp)
    lo, hi = domain(mp)
    rng = np.random.default_rng(seed)
    pts = rng.uniform(lo, hi, size=(n, 3))
    return mp, om, pts, rng


def _p2g_loss(oracle, om, mp, pts, order, kind, x, gbar):
    grid = np.zeros(mp.extents() + (P2G_DOFS[kind],))
    assert oracle.p2g(om, pts, order, [(kind, -0.7, x, grid)]) == 0
    return float((grid * gbar).sum())


def _g2p_loss(oracle, om, pts, order, kind, grid, xbar):
    out = np.zeros((pts.shape[0], G2P_COMPS[kind]))
    assert oracle.g2p(om, pts, order, [(kind, 1.3, out, grid.copy())]) == 0
    return float((out * xbar).sum())


def _fd_positions(loss, pts, step):
    fd = np.zeros_like(pts)
    for p in range(pts.shape[0]):
        for e in range(3):
            a = pts.copy()
            b = pts.copy()
            a[p, e] += step
            b[p, e] -= step
            fd[p, e] = (loss(a) - loss(b)) / (2 * step)
    return fd


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("kind", range(6))
def test_p2g_adjoint_against_differences(oracle, kind, order, periodic):
    mp, om, pts, rng = _setup(oracle, order, periodic, 100 * kind + order)
    x = rng.normal(size=(pts.shape[0], P2G_COMPS[kind]))
    gbar = rng.normal(size=mp.extents() + (P2G_DOFS[kind],))
    xbar = np.zeros_like(x)
    pbar = np.zeros_like(pts)
    op = dict(kind=kind, mult=-0.7, x=x, x_bar=xbar, array_bar=gbar.copy())
    assert oracle.p2g_adjoint(om, pts, order, [op], points_bar=pbar) == 0
    # positions: central difference of the forward loss
    fd = _fd_positions(lambda q: _p2g_loss(oracle, om, mp, q, order, kind, x, gbar), pts, 1e-5)
    scale = max(np.abs(fd).max(), 1e-300)
    assert np.abs(pbar - fd).max() <= 1e-6 * scale
    # point field: the loss is linear in x
    dx = rng.normal(size=x.shape)
    dl = _p2g_loss(oracle, om, mp, pts, order, kind, x + dx, gbar) - _p2g_loss(oracle, om, mp, pts, order, kind, x, gbar)
    assert abs((xbar * dx).sum() - dl) <= 1e-10 * max(abs(dl), np.abs(xbar).sum())


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("kind", range(6))
def test_g2p_adjoint_against_differences(oracle, kind, order, periodic):
    mp, om, pts, rng = _setup(oracle, order, periodic, 200 * kind + order)
    grid = rng.normal(size=mp.extents() + (G2P_DOFS[kind],))
    oracle.halo_gather(om, grid)  # the forward array as g2p reads it
    xbar = rng.normal(size=(pts.shape[0], G2P_COMPS[kind]))
    gbar = np.zeros_like(grid)
    pbar = np.zeros_like(pts)
    op = dict(kind=kind, mult=1.3, x_bar=xbar, array=grid, array_bar=gbar)
    assert oracle.g2p_adjoint(om, pts, order, [op], points_bar=pbar) == 0
    fd = _fd_positions(lambda q: _g2p_loss(oracle, om, q, order, kind, grid, xbar), pts, 1e-5)
    scale = max(np.abs(fd).max(), 1e-300)
    assert np.abs(pbar - fd).max() <= 1e-6 * scale
    # grid: the loss is linear in the array (the forward's halo gather included)
    dg = rng.normal(size=grid.shape)
    dl = _g2p_loss(oracle, om, pts, order, kind, grid + dg, xbar) - _g2p_loss(oracle, om, pts, order, kind, grid, xbar)
    assert abs((gbar * dg).sum() - dl) <= 1e-10 * max(abs(dl), np.abs(gbar).sum())
