"""Known-answer tests that pin the oracle's 2D p2g / g2p restatement.

* grid/unit_test/tstInterpolation2d.hpp: periodic 2D mesh, one point at every
  cell centre, Spline<1>, constant fields 3.5 and multiplier -0.5 give -1.75
  on every owned node (value operators) and 0 (gradient / divergence
  operators), and the same numbers back on the points after g2p.
* grid/unit_test/tstSplineEvaluation2d.hpp: cell-centred points, Spline<1> on
  nodes: cell size 0.05, logical coordinates i + 0.5, stencil {i, i+1},
  weights 0.5, gradient-weight products +-0.5 / dx, sum of w * d = 0.
* The 2D operators against the 3D ones (themselves pinned by the 3D tests):
  a 3D mesh with the same (i, j) layout, summed over k, equals the 2D result
  for every operator that does not differentiate along k (the k weights sum
  to one).
"""
import numpy as np
import pytest

from cabana_gb300 import mesh as M
from tests.conftest import float_eq

P2G_COMPS_2D = {0: 1, 1: 2, 2: 1, 3: 2, 4: 4}
P2G_DOFS_2D = {0: 1, 1: 2, 2: 2, 3: 1, 4: 2}
G2P_COMPS_2D = {0: 1, 1: 2, 2: 2, 3: 4, 4: 1}
G2P_DOFS_2D = {0: 1, 1: 2, 2: 1, 3: 2, 4: 2}


def _mesh2(oracle, lg, entity=M.NODE):
    mp = M.mesh_params(lg, entity)
    assert mp.num_space_dim == 2
    return mp, oracle.make_mesh(mp.ghost_low, mp.cell_size, mp.owned_cells, mp.halo_width, mp.periodic, mp.entity,
                                num_space_dim=2)


def _cell_centres(lg, lm):
    (i0, i1), (j0, j1) = lg.ownedSpace(M.CELL)
    # pid = pi + ni * pj: i fastest (tstInterpolation2d.hpp fill_points)
    return np.array([lm.coordinates(M.CELL, (i, j)) for j in range(j0, j1) for i in range(i0, i1)], np.float64)


@pytest.fixture(scope="module")
def periodic2d(oracle):
    gm = M.createUniformGlobalMesh((-1.2, 0.1), (-0.2, 9.5), 0.1)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, (True, True)), 1)
    lm = M.createLocalMesh(lg)
    mp, om = _mesh2(oracle, lg)
    return lg, lm, mp, om, _cell_centres(lg, lm)


def test_mesh_is_2d(periodic2d, oracle):
    lg, lm, mp, om, pts = periodic2d
    assert pts.shape[1] == 2
    assert oracle.extents(om) == mp.extents() == (13, 97)   # 10 and 94 cells + 2 halo + 1 (nodes)
    assert lg.ownedSpace(M.NODE) == ((1, 11), (1, 95))


def test_p2g_constants_2d(oracle, periodic2d):
    lg, lm, mp, om, pts = periodic2d
    n = pts.shape[0]
    ext = mp.extents()
    (i0, i1), (j0, j1) = lg.ownedSpace(M.NODE)
    cases = [(0, 1, -1.75), (1, 2, -1.75), (2, 2, 0.0), (3, 1, 0.0), (4, 2, 0.0)]
    for kind, dofs, expect in cases:
        x = np.full((n, P2G_COMPS_2D[kind]), 3.5)
        grid = np.zeros(ext + (dofs,))
        assert oracle.p2g(om, pts, 1, [(kind, -0.5, x, grid)]) == 0
        owned = grid[i0:i1, j0:j1]
        if expect == 0.0:
            assert all(float_eq(v + 1.0, 1.0) for v in owned.ravel())
        else:
            assert all(float_eq(v, expect) for v in owned.ravel())


def test_g2p_constants_2d(oracle, periodic2d):
    lg, lm, mp, om, pts = periodic2d
    n = pts.shape[0]
    ext = mp.extents()
    (i0, i1), (j0, j1) = lg.ownedSpace(M.NODE)
    scalar_grid = np.zeros(ext + (1,))
    vector_grid = np.zeros(ext + (2,))
    scalar_grid[i0:i1, j0:j1] = 3.5   # ArrayOp::assign(..., 3.5, Own())
    vector_grid[i0:i1, j0:j1] = 3.5
    cases = [(0, scalar_grid, -1.75), (1, vector_grid, -1.75), (2, scalar_grid, 0.0), (3, vector_grid, 0.0),
             (4, vector_grid, 0.0)]
    for kind, grid, expect in cases:
        x = np.zeros((n, G2P_COMPS_2D[kind]))
        assert oracle.g2p(om, pts, 1, [(kind, -0.5, x, grid.copy())]) == 0
        if expect == 0.0:
            assert all(float_eq(v + 1.0, 1.0) for v in x.ravel())
        else:
            assert all(float_eq(v, expect) for v in x.ravel())


def test_spline_evaluation_cell_centres_2d(oracle):
    gm = M.createUniformGlobalMesh((-1.2, 0.1), (-0.3, 9.5), 0.05)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, (True, True)), 1)
    lm = M.createLocalMesh(lg)
    mp, om = _mesh2(oracle, lg)
    (i0, i1), (j0, j1) = lg.ownedSpace(M.CELL)
    rng = np.random.default_rng(7)
    for _ in range(200):
        idx = (int(rng.integers(i0, i1)), int(rng.integers(j0, j1)))
        p = lm.coordinates(M.CELL, idx)
        sd = oracle.evaluate_spline(om, 1, p)
        for d in range(2):
            assert float_eq(sd["dx"][d], 0.05)
            assert float_eq(sd["x"][d], idx[d] + 0.5)
            assert list(sd["s"][d]) == [idx[d], idx[d] + 1]
            assert float_eq(sd["w"][d][0], 0.5) and float_eq(sd["w"][d][1], 0.5)
            assert float_eq((sd["w"][d] * sd["d"][d]).sum() + 1.0, 1.0)
        # gradient (i, j) products of tstSplineEvaluation2d.hpp: g_i w_j
        for (a, b), sx, sy in [((0, 0), -1, -1), ((1, 0), 1, -1), ((1, 1), 1, 1), ((0, 1), -1, 1)]:
            assert float_eq(sd["g"][0][a] * sd["w"][1][b], sx * 0.5 / 0.05)
            assert float_eq(sd["w"][0][a] * sd["g"][1][b], sy * 0.5 / 0.05)


def test_nonperiodic_halo_is_noop_2d(oracle):
    gm = M.createUniformGlobalMesh((0.0, 1.0), (3.0, 5.0), 0.5)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, (False, False)), 2)
    mp, om = _mesh2(oracle, lg)
    a = np.random.default_rng(0).normal(size=mp.extents() + (2,))
    b = a.copy()
    oracle.halo_scatter_sum(om, b)
    oracle.halo_gather(om, b)
    np.testing.assert_array_equal(a, b)


def test_periodic_fold_conserves_2d(oracle):
    gm = M.createUniformGlobalMesh((0.0, 0.0), (4.0, 3.0), 0.5)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, (True, False)), 2)
    mp, om = _mesh2(oracle, lg)
    rng = np.random.default_rng(4)
    n = 500
    # any x (the fold wraps it), y away from the non-periodic ends so every
    # stencil stays in owned j rows
    pts = np.stack([rng.uniform(0.0, 4.0, n), rng.uniform(1.0, 2.0, n)], axis=1)
    m = rng.uniform(0.5, 1.5, size=(n, 1))
    for order in (1, 2, 3):
        grid = np.zeros(mp.extents() + (1,))
        assert oracle.p2g(om, pts, order, [(0, 1.0, m, grid)]) == 0
        (i0, i1), (j0, j1) = lg.ownedSpace(M.NODE)
        # after scatter(Sum) the owned nodes (periodic in i) carry all the mass
        assert abs(grid[i0:i1, j0:j1].sum() - m.sum()) < 1e-12 * m.sum()
        # and the i ghosts still hold their copies (scatter does not clear them)
        assert grid[:i0].sum() + grid[i1:].sum() > 0.0


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5, 6])
def test_2d_matches_3d_summed_over_k(oracle, order):
    """2D operators = 3D operators summed over k, for every operator that does
    not differentiate along k: the 3D stencil's k weights sum to one."""
    lo2, hi2 = (-0.4, 1.3), (-0.4 + 9 * 0.3, 1.3 + 7 * 0.3)
    gm2 = M.createUniformGlobalMesh(lo2, hi2, 0.3)
    lg2 = M.createLocalGrid(M.createGlobalGrid(gm2, (False, False)), 4)
    mp2, om2 = _mesh2(oracle, lg2)
    gm3 = M.createUniformGlobalMesh(lo2 + (0.0,), hi2 + (12 * 0.3,), 0.3)
    lg3 = M.createLocalGrid(M.createGlobalGrid(gm3, (False, False, False)), 4)
    mp3 = M.mesh_params(lg3)
    om3 = oracle.make_mesh(mp3.ghost_low, mp3.cell_size, mp3.owned_cells, mp3.halo_width, mp3.periodic, mp3.entity)
    rng = np.random.default_rng(100 + order)
    n = 400
    p2 = np.stack([rng.uniform(lo2[0], hi2[0], n), rng.uniform(lo2[1], hi2[1], n)], axis=1)
    p3 = np.concatenate([p2, rng.uniform(1.2, 2.4, size=(n, 1))], axis=1)
    # P2G: ScalarValue, ScalarGradient (dofs 0, 1 = d/dx, d/dy)
    s = rng.normal(size=(n, 1))
    for kind, dofs2, dofs3, take in [(0, 1, 1, [0]), (2, 2, 3, [0, 1])]:
        g2 = np.zeros(mp2.extents() + (dofs2,))
        g3 = np.zeros(mp3.extents() + (dofs3,))
        assert oracle.p2g(om2, p2, order, [(kind, 0.7, s, g2)]) == 0
        assert oracle.p2g(om3, p3, order, [(kind, 0.7, s, g3)]) == 0
        np.testing.assert_allclose(g3.sum(axis=2)[..., take], g2, rtol=1e-12, atol=1e-12)
    # VectorValue P2G: 3D vector with a zero z component
    v = rng.normal(size=(n, 2))
    g2 = np.zeros(mp2.extents() + (2,))
    g3 = np.zeros(mp3.extents() + (3,))
    assert oracle.p2g(om2, p2, order, [(1, -1.1, v, g2)]) == 0
    assert oracle.p2g(om3, p3, order, [(1, -1.1, np.concatenate([v, np.zeros((n, 1))], 1), g3)]) == 0
    np.testing.assert_allclose(g3.sum(axis=2)[..., :2], g2, rtol=1e-12, atol=1e-12)
    # G2P from a grid constant along k: ScalarValue, ScalarGradient (x, y)
    f2 = rng.normal(size=mp2.extents() + (1,))
    f3 = np.repeat(f2[:, :, None, :], mp3.extents()[2], axis=2).copy()
    for kind, c2, c3, take in [(0, 1, 1, [0]), (2, 2, 3, [0, 1])]:
        x2 = np.zeros((n, c2))
        x3 = np.zeros((n, c3))
        assert oracle.g2p(om2, p2, order, [(kind, 0.9, x2, f2.copy())]) == 0
        assert oracle.g2p(om3, p3, order, [(kind, 0.9, x3, f3.copy())]) == 0
        np.testing.assert_allclose(x3[:, take], x2, rtol=1e-11, atol=1e-12)
