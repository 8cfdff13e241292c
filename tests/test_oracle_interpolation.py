"""Known-answer tests that pin the oracle's p2g / g2p restatement.

* grid/unit_test/tstInterpolation3d.hpp:38-251: periodic mesh, one point at
  every cell centre, Spline<1>, constant fields 3.5 and multiplier -0.5 give
  -1.75 on every owned node (value operators) and 0 (gradient / divergence
  operators), and the same numbers back on the points after g2p.
* grid/unit_test/tstSplineEvaluation3d.hpp:262-511: cell-centred points,
  Spline<1> on nodes: cell size, logical coordinates i + 0.5, stencil
  {i, i+1}, weights 0.5, gradient weights +-1/(2 dx), sum of w*d = 0.
* The 1-D identities of grid/unit_test/tstSplines.cpp (partition of unity,
  linear reproduction and its derivative) lifted to the 3D operators on
  random points, Spline<0..6>: P2G moments and G2P of linear grid fields.
"""
import numpy as np
import pytest

from cabana_gb300 import mesh as M
from tests.conftest import float_eq


def _cell_centre_points(lg, lm):
    (i0, i1), (j0, j1), (k0, k1) = lg.ownedSpace(M.CELL)
    pts = []
    # pid = pi + ni * (pj + nj * pk): i fastest (tstInterpolation3d.hpp:62-75)
    for k in range(k0, k1):
        for j in range(j0, j1):
            for i in range(i0, i1):
                pts.append(lm.coordinates(M.CELL, (i, j, k)))
    return np.array(pts, np.float64)


@pytest.fixture(scope="module")
def periodic_setup(oracle):
    gm = M.createUniformGlobalMesh((-1.2, 0.1, 1.1), (-0.3, 9.5, 2.3), 0.1)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, (True, True, True)), 1)
    lm = M.createLocalMesh(lg)
    mp = M.mesh_params(lg, M.NODE)
    om = oracle.make_mesh(mp.ghost_low, mp.cell_size, mp.owned_cells, mp.halo_width, mp.periodic, mp.entity)
    return lg, lm, mp, om, _cell_centre_points(lg, lm)


def _owned(lg, a):
    (i0, i1), (j0, j1), (k0, k1) = lg.ownedSpace(M.NODE)
    return a[i0:i1, j0:j1, k0:k1]


def test_p2g_constants(oracle, periodic_setup):
    lg, lm, mp, om, pts = periodic_setup
    n = pts.shape[0]
    ext = mp.extents()
    scalar_pt = np.full((n, 1), 3.5)
    vector_pt = np.full((n, 3), 3.5)
    tensor_pt = np.full((n, 9), 3.5)
    cases = [(0, scalar_pt, 1, -1.75), (1, vector_pt, 3, -1.75), (2, scalar_pt, 3, 0.0),
             (3, vector_pt, 1, 0.0), (4, tensor_pt, 3, 0.0)]
    for kind, x, dofs, expect in cases:
        grid = np.zeros(ext + (dofs,))
        assert oracle.p2g(om, pts, 1, [(kind, -0.5, x, grid)]) == 0
        owned = _owned(lg, grid)
        if expect == 0.0:
            assert all(float_eq(v + 1.0, 1.0) for v in owned.ravel())
        else:
            assert all(float_eq(v, expect) for v in owned.ravel())


def test_g2p_constants(oracle, periodic_setup):
    lg, lm, mp, om, pts = periodic_setup
    n = pts.shape[0]
    ext = mp.extents()
    scalar_grid = np.zeros(ext + (1,))
    vector_grid = np.zeros(ext + (3,))
    (i0, i1), (j0, j1), (k0, k1) = lg.ownedSpace(M.NODE)
    scalar_grid[i0:i1, j0:j1, k0:k1] = 3.5   # ArrayOp::assign(..., 3.5, Own())
    vector_grid[i0:i1, j0:j1, k0:k1] = 3.5
    cases = [(0, scalar_grid, 1, -1.75), (1, vector_grid, 3, -1.75), (2, scalar_grid, 3, 0.0),
             (3, vector_grid, 9, 0.0), (4, vector_grid, 1, 0.0)]
    for kind, grid, comps, expect in cases:
        x = np.zeros((n, comps))
        assert oracle.g2p(om, pts, 1, [(kind, -0.5, x, grid)]) == 0
        if expect == 0.0:
            assert all(float_eq(v + 1.0, 1.0) for v in x.ravel())
        else:
            assert all(float_eq(v, expect) for v in x.ravel())


def test_spline_evaluation_cell_centres(oracle):
    gm = M.createUniformGlobalMesh((-1.2, 0.1, 1.1), (-0.3, 9.5, 2.3), 0.05)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, (True, True, True)), 1)
    lm = M.createLocalMesh(lg)
    mp = M.mesh_params(lg, M.NODE)
    om = oracle.make_mesh(mp.ghost_low, mp.cell_size, mp.owned_cells, mp.halo_width, mp.periodic, mp.entity)
    (i0, i1), (j0, j1), (k0, k1) = lg.ownedSpace(M.CELL)
    rng = np.random.default_rng(7)
    for _ in range(200):
        idx = (rng.integers(i0, i1), rng.integers(j0, j1), rng.integers(k0, k1))
        p = lm.coordinates(M.CELL, idx)
        sd = oracle.evaluate_spline(om, 1, p)
        for d in range(3):
            assert float_eq(sd["dx"][d], 0.05)
            assert float_eq(sd["x"][d], idx[d] + 0.5)
            assert list(sd["s"][d]) == [idx[d], idx[d] + 1]
            assert float_eq(sd["w"][d][0], 0.5) and float_eq(sd["w"][d][1], 0.5)
            assert float_eq(sd["g"][d][0], -1.0 / 0.05) and float_eq(sd["g"][d][1], 1.0 / 0.05)
            # sum_n w * d == 0 (the point sits half way between its knots)
            assert float_eq((sd["w"][d] * sd["d"][d]).sum() + 1.0, 1.0)
        # gradient-weight products: g_i w_j w_k = +-0.25 / dx
        prod = sd["g"][0][0] * sd["w"][1][0] * sd["w"][2][0]
        assert float_eq(prod, -0.25 / 0.05)


def test_nonperiodic_halo_is_noop(oracle):
    lg, mp = M.simple_mesh(6, 0.5, (1.0, -2.0, 0.25), 2)
    om = oracle.make_mesh(mp.ghost_low, mp.cell_size, mp.owned_cells, mp.halo_width, mp.periodic, mp.entity)
    a = np.random.default_rng(0).normal(size=mp.extents() + (3,))
    b = a.copy()
    oracle.halo_scatter_sum(om, b)
    oracle.halo_gather(om, b)
    np.testing.assert_array_equal(a, b)


def test_openmp_duplicated_scatter_matches_serial(oracle):
    lg, mp = M.simple_mesh(8, 1.0)
    om = oracle.make_mesh(mp.ghost_low, mp.cell_size, mp.owned_cells, mp.halo_width, mp.periodic, mp.entity)
    rng = np.random.default_rng(3)
    n = 5000
    pts = rng.uniform(0.0, 8.0, size=(n, 3))
    m = rng.uniform(0.5, 1.5, size=(n, 1))
    for order in (1, 2, 3):
        g1 = np.zeros(mp.extents() + (1,))
        g4 = np.zeros(mp.extents() + (1,))
        oracle.p2g(om, pts, order, [(0, 1.0, m, g1)], nthreads=1)
        oracle.p2g(om, pts, order, [(0, 1.0, m, g4)], nthreads=4)
        np.testing.assert_allclose(g4, g1, rtol=1e-13, atol=1e-13)
        assert abs(g1.sum() - m.sum()) < 1e-9 * m.sum()


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5, 6])
def test_p2g_moments_random_points(oracle, order):
    """B-spline identities at the operator level on random (not cell-centred)
    points: ScalarValueP2G of ones sums to the particle count (partition of
    unity) and its node-coordinate moments give the particle positions (linear
    reproduction, orders >= 1); ScalarGradientP2G of ones sums to zero and its
    moments give the identity (the derivative of linear reproduction). They pin
    which node and which dof each weight product lands on in 3D."""
    lg, mp = M.simple_mesh((9, 7, 8), 0.3, (0.4, -1.3, 2.0), 4)
    om = oracle.make_mesh(mp.ghost_low, mp.cell_size, mp.owned_cells, mp.halo_width, mp.periodic, mp.entity)
    rng = np.random.default_rng(40 + order)
    n = 2000
    lo = np.array((0.4, -1.3, 2.0))
    pts = lo + rng.uniform(0.0, 1.0, size=(n, 3)) * (np.array((9, 7, 8)) * 0.3)
    ext = mp.extents()
    coords = [np.asarray(mp.ghost_low[d]) + np.arange(ext[d]) * mp.cell_size[d] for d in range(3)]
    X = np.stack(np.meshgrid(*coords, indexing="ij"), axis=-1)  # node coordinates (i, j, k, d)
    ones = np.ones((n, 1))
    value = np.zeros(ext + (1,))
    assert oracle.p2g(om, pts, order, [(0, 1.0, ones, value)]) == 0
    assert abs(value.sum() - n) < 1e-10 * n
    if order >= 1:
        moments = np.einsum("ijk,ijkd->d", value[..., 0], X)
        np.testing.assert_allclose(moments, pts.sum(axis=0), rtol=1e-12)
    grad = np.zeros(ext + (3,))
    assert oracle.p2g(om, pts, order, [(2, 1.0, ones, grad)]) == 0
    np.testing.assert_allclose(grad.sum(axis=(0, 1, 2)), 0.0, atol=1e-9 * n / 0.3)
    if order >= 1:
        jac = np.einsum("ijkd,ijke->de", grad, X)  # sum over particles of d x_e / d x_d
        np.testing.assert_allclose(jac, n * np.eye(3), atol=1e-8 * n)


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6])
def test_g2p_reproduces_linear_fields(oracle, order):
    """G2P of a grid field that is linear in the node coordinates, f = a . X +
    b: ScalarValueG2P returns f(x_p) and ScalarGradientG2P returns a at every
    random point; VectorGradientG2P of (f, 2 f, -f) returns the rows
    (derivative index first, as Interpolation.hpp:247-282) a x (1, 2, -1)."""
    lg, mp = M.simple_mesh((9, 7, 8), 0.3, (0.4, -1.3, 2.0), 4)
    om = oracle.make_mesh(mp.ghost_low, mp.cell_size, mp.owned_cells, mp.halo_width, mp.periodic, mp.entity)
    rng = np.random.default_rng(60 + order)
    n = 1500
    lo = np.array((0.4, -1.3, 2.0))
    pts = lo + rng.uniform(0.0, 1.0, size=(n, 3)) * (np.array((9, 7, 8)) * 0.3)
    ext = mp.extents()
    coords = [np.asarray(mp.ghost_low[d]) + np.arange(ext[d]) * mp.cell_size[d] for d in range(3)]
    X = np.stack(np.meshgrid(*coords, indexing="ij"), axis=-1)
    a, b = np.array((0.7, -1.9, 2.6)), 0.35
    f = (X @ a + b)[..., None]
    val = np.zeros((n, 1))
    assert oracle.g2p(om, pts, order, [(0, 1.0, val, f.copy())]) == 0
    np.testing.assert_allclose(val[:, 0], pts @ a + b, rtol=1e-11, atol=1e-11)
    grad = np.zeros((n, 3))
    assert oracle.g2p(om, pts, order, [(2, 1.0, grad, f.copy())]) == 0
    np.testing.assert_allclose(grad, np.broadcast_to(a, (n, 3)), rtol=1e-10, atol=1e-10)
    fv = np.concatenate([f, 2.0 * f, -f], axis=-1)
    vg = np.zeros((n, 9))
    assert oracle.g2p(om, pts, order, [(3, 1.0, vg, fv)]) == 0
    expect = np.outer(a, (1.0, 2.0, -1.0)).ravel()  # result[m][n] = sum d_m W f_n
    np.testing.assert_allclose(vg, np.broadcast_to(expect, (n, 9)), rtol=1e-10, atol=1e-10)
