"""The oracle's fused g2p2g (benchmark/grid/Cabana_Grid_InterpolationPerformance.cpp:
129-174, with G2P reading each array as it was at the call), pinned by:

* the reference's own constants (tstInterpolation3d.hpp:38-251 setup:
  periodic mesh, one point per cell centre, Spline<1>, an owned field of 3.5):
  ScalarValueG2P(-0.5) gives -1.75 on every point, and ScalarValueP2G(-0.5)
  of that into the same array adds 0.875 to every owned node away from the
  periodic seams (there the scatter(Sum) also folds in the ghost values that
  the gather copied, as the reference's composition does);
* the sequential composition g2p then p2g, which it must equal exactly when
  no array is both read and written, and equal with a copy of the read array
  when one is.
"""
import numpy as np
import pytest

from cabana_gb300 import mesh as M
from tests.conftest import float_eq
from tests.helpers import oracle_mesh


def _periodic(oracle):
    gm = M.createUniformGlobalMesh((-1.2, 0.1, 1.1), (-0.3, 9.5, 2.3), 0.1)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, (True, True, True)), 1)
    lm = M.createLocalMesh(lg)
    mp = M.mesh_params(lg)
    (i0, i1), (j0, j1), (k0, k1) = lg.ownedSpace(M.CELL)
    pts = np.array([lm.coordinates(M.CELL, (i, j, k)) for k in range(k0, k1) for j in range(j0, j1)
                    for i in range(i0, i1)])
    return lg, mp, oracle_mesh(oracle, mp), pts


def test_reference_scalar_g2p2g_constants(oracle):
    lg, mp, om, pts = _periodic(oracle)
    n = pts.shape[0]
    own = tuple(slice(a, b) for a, b in lg.ownedSpace(M.NODE))
    grid = np.zeros(mp.extents() + (1,))
    grid[own] = 3.5
    scalar = np.zeros((n, 1))
    assert oracle.g2p2g(om, pts, 1, [(0, -0.5, scalar, grid)], [(0, -0.5, scalar, grid)]) == 0
    assert all(float_eq(v, -1.75) for v in scalar.ravel())
    (i0, i1), (j0, j1), (k0, k1) = lg.ownedSpace(M.NODE)
    # owned nodes without a ghost image (the ghost layers are hw below and
    # hw + 1 above the owned range in every periodic dimension)
    inner = grid[i0 + 2:i1 - 1, j0 + 2:j1 - 1, k0 + 2:k1 - 1]
    assert inner.size > 0 and all(float_eq(v, 3.5 + 0.875) for v in inner.ravel())
    # every ghost has an owned image on this fully periodic mesh: the owned
    # total is every node's gathered 3.5 plus the points' 0.875 each
    total = 3.5 * int(np.prod(mp.extents())) + 0.875 * n
    assert abs(grid[own].sum() - total) < 1e-9 * total


def _random_case(oracle, seed, order):
    lg, mp = M.simple_mesh(7, 0.6, (0.4, -1.0, 2.0), 3)
    om = oracle_mesh(oracle, mp)
    rng = np.random.default_rng(seed)
    n = 700
    lo = np.array(mp.ghost_low) + 3 * 0.6
    pts = lo + rng.uniform(0.0, 7 * 0.6, size=(n, 3))
    return mp, om, pts, rng, n


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4])
def test_equals_sequential_composition(oracle, order):
    mp, om, pts, rng, n = _random_case(oracle, 40 + order, order)
    ext = mp.extents()
    mom = rng.normal(size=ext + (3,))
    sgrid = rng.normal(size=ext + (1,))
    vel0 = rng.normal(size=(n, 3))
    s0 = rng.normal(size=(n, 1))
    # fused: velocity from the momentum grid, scalar from the scalar grid, then
    # momentum-like P2G of the new velocity into a fresh grid and the scalar
    # back into its own grid (read from the state at the call)
    vel, s, out, sg = vel0.copy(), s0.copy(), np.zeros(ext + (3,)), sgrid.copy()
    assert oracle.g2p2g(om, pts, order, [(1, 0.8, vel, mom.copy()), (0, -0.5, s, sg)],
                        [(1, 1.3, vel, out), (0, -0.5, s, sg)]) == 0
    # sequential: g2p on copies, then p2g
    vel2, s2, out2, sg2 = vel0.copy(), s0.copy(), np.zeros(ext + (3,)), sgrid.copy()
    assert oracle.g2p(om, pts, order, [(1, 0.8, vel2, mom.copy()), (0, -0.5, s2, sgrid.copy())]) == 0
    assert oracle.p2g(om, pts, order, [(1, 1.3, vel2, out2), (0, -0.5, s2, sg2)]) == 0
    np.testing.assert_array_equal(vel, vel2)
    np.testing.assert_array_equal(s, s2)
    np.testing.assert_array_equal(out, out2)
    np.testing.assert_array_equal(sg, sg2)
