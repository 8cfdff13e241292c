"""GPU parity of the fused g2p2g (cgx_g2p2g) against the FP64 oracle.

Tolerances (max|gpu - oracle| / max|oracle|): CGX_PLAIN_FP64 1e-12;
CGX_FP32_COMPENSATED point fields 4e-6, grids 4e-6 (plain float atomics).
"""
import numpy as np
import pytest
import torch

from cabana_gb300 import grid as G
from cabana_gb300 import mesh as M
from tests.helpers import max_rel, oracle_mesh

pytestmark = pytest.mark.gpu

FORMS = [("plain64", G.PLAIN_FP64), ("fp32", G.FP32_COMPENSATED)]


@pytest.mark.parametrize("form_name,precision", FORMS)
def test_reference_scalar_g2p2g(oracle, form_name, precision):
    """The reference benchmark's scalar g2p2g on the tstInterpolation3d
    constants: one array read by ScalarValueG2P(-0.5) and written by
    ScalarValueP2G(-0.5), periodic, Spline<1>."""
    gm = M.createUniformGlobalMesh((-1.2, 0.1, 1.1), (-0.3, 9.5, 2.3), 0.1)
    lg = M.createLocalGrid(M.createGlobalGrid(gm, (True, True, True)), 1)
    lm = M.createLocalMesh(lg)
    mp = M.mesh_params(lg)
    (i0, i1), (j0, j1), (k0, k1) = lg.ownedSpace(M.CELL)
    pts = np.array([lm.coordinates(M.CELL, (i, j, k)) for k in range(k0, k1) for j in range(j0, j1)
                    for i in range(i0, i1)])
    n = pts.shape[0]
    ref = np.zeros(mp.extents() + (1,))
    own = tuple(slice(a, b) for a, b in lg.ownedSpace(M.NODE))
    ref[own] = 3.5
    s_ref = np.zeros((n, 1))
    assert oracle.g2p2g(oracle_mesh(oracle, mp), pts, 1, [(0, -0.5, s_ref, ref)], [(0, -0.5, s_ref, ref)]) == 0
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    arr = G.createArray("s", G.createArrayLayout(lg, 1, M.Node), dt)
    G.ArrayOp.assign(arr, 3.5, G.Own)
    scalar = torch.zeros(n, dtype=dt, device="cuda")
    G.g2p2g(G.createScalarValueP2G(scalar, -0.5), torch.tensor(pts, device="cuda"), n, G.Spline(1),
            G.createHalo(G.NodeHaloPattern(), 1), arr, G.createScalarValueG2P(scalar, -0.5), precision=precision)
    tol = 1e-12 if precision == G.PLAIN_FP64 else 4e-6
    assert max_rel(scalar.double().cpu().numpy(), s_ref[:, 0]) <= tol
    assert max_rel(arr.view().double().cpu().numpy(), ref) <= tol


@pytest.mark.parametrize("form_name,precision", FORMS)
@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5, 6])
def test_mpm_style_g2p2g_vs_oracle(oracle, form_name, precision, order):
    """Velocity and its gradient from a momentum grid, then mass, momentum
    of the new velocity and a stress divergence into other arrays, plus a
    scalar read and written in place; one launch."""
    lg, mp = M.simple_mesh((9, 7, 8), 0.45, (0.3, -1.1, 2.0), 3, periodic=(True, False, False))
    om = oracle_mesh(oracle, mp)
    rng = np.random.default_rng(900 + order)
    n = 4000
    lo = np.array(mp.ghost_low) + 3 * 0.45
    pts = lo + rng.uniform(0.0, 1.0, size=(n, 3)) * (np.array((9, 7, 8)) * 0.45)
    pts[:, 1:] = np.clip(pts[:, 1:], lo[1:] + 0.2, lo[1:] + np.array((7, 8)) * 0.45 - 0.2)
    ext = mp.extents()
    mom = rng.normal(size=ext + (3,))
    sgrid = rng.normal(size=ext + (1,))
    vel0 = rng.normal(size=(n, 3))
    vg0 = rng.normal(size=(n, 9))
    s0 = rng.normal(size=(n, 1))
    mass = rng.uniform(0.5, 1.5, size=(n, 1))
    stress = rng.normal(size=(n, 9))
    r_vel, r_vg, r_s = vel0.copy(), vg0.copy(), s0.copy()
    r_mass, r_mom2, r_frc, r_sg = (np.zeros(ext + (1,)), np.zeros(ext + (3,)), np.zeros(ext + (3,)), sgrid.copy())
    r_momsrc = mom.copy()
    assert oracle.g2p2g(om, pts, order,
                        [(1, 1.0, r_vel, r_momsrc), (3, 0.5, r_vg, r_momsrc), (0, -0.5, r_s, r_sg)],
                        [(0, 1.0, mass, r_mass), (1, 0.7, r_vel, r_mom2), (4, -1.0, stress, r_frc),
                         (0, -0.5, r_s, r_sg)]) == 0
    dt = torch.float64 if precision == G.PLAIN_FP64 else torch.float32
    cu = lambda a, shape=None: torch.tensor(a, device="cuda").to(dt).reshape(shape or a.shape).contiguous()  # noqa: E731
    vel, vg, s = cu(vel0), cu(vg0, (n, 3, 3)), cu(s0, (n,))
    tmass, tstress = cu(mass, (n,)), cu(stress, (n, 3, 3))
    lay = lambda d: G.createArrayLayout(lg, d, M.Node)  # noqa: E731
    a_mom = G.createArray("mom", lay(3), dt)
    a_mom.view().copy_(cu(mom))
    a_s = G.createArray("s", lay(1), dt)
    a_s.view().copy_(cu(sgrid))
    a_mass, a_mom2, a_frc = G.createArray("m", lay(1), dt), G.createArray("p", lay(3), dt), G.createArray("f", lay(3), dt)
    G.g2p2g([G.createScalarValueP2G(tmass, 1.0), G.createVectorValueP2G(vel, 0.7),
             G.createTensorDivergenceP2G(tstress, -1.0), G.createScalarValueP2G(s, -0.5)],
            torch.tensor(pts, device="cuda"), n, G.Spline(order), G.createHalo(G.NodeHaloPattern(), 3),
            [a_mass, a_mom2, a_frc, a_s],
            [G.createVectorValueG2P(vel, 1.0), G.createVectorGradientG2P(vg, 0.5), G.createScalarValueG2P(s, -0.5)],
            [a_mom, a_mom, a_s], precision=precision, check_bounds=True)
    assert G.last_dispatch() == "points"
    tol = 1e-12 if precision == G.PLAIN_FP64 else 4e-6
    for got, ref in [(vel, r_vel), (vg.reshape(n, 9), r_vg), (s.reshape(n, 1), r_s), (a_mass.view(), r_mass),
                     (a_mom2.view(), r_mom2), (a_frc.view(), r_frc), (a_s.view(), r_sg)]:
        assert max_rel(got.double().cpu().numpy(), ref) <= tol, (form_name, order)
    # the read array is left as it was (no functor writes it)
    assert max_rel(a_mom.view().double().cpu().numpy(), r_momsrc) <= (1e-15 if precision == G.PLAIN_FP64 else 1e-7)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_tiled_g2p2g_vs_oracle(oracle, order):
    """With a tiling and the FP32 form, cgx_g2p2g runs the tiled G2P then the
    tiled P2G launch: the same contract (G2P reads the state at the call)."""
    from cabana_gb300 import core
    lg, mp = M.simple_mesh((10, 9, 8), 0.5, (0.3, -1.1, 2.0), 2)
    om = oracle_mesh(oracle, mp)
    rng = np.random.default_rng(1200 + order)
    n = 20000
    lo = np.array(mp.ghost_low) + 2 * 0.5
    pts = lo + rng.uniform(0.0, 1.0, size=(n, 3)) * (np.array((10, 9, 8)) * 0.5)
    ext = mp.extents()
    mom = rng.normal(size=ext + (3,))
    sgrid = rng.normal(size=ext + (1,))
    vel0 = rng.normal(size=(n, 3))
    s0 = rng.normal(size=(n, 1))
    mass = rng.uniform(0.5, 1.5, size=(n, 1))
    r_vel, r_s, r_mass, r_mom2, r_sg, r_mom = (vel0.copy(), s0.copy(), np.zeros(ext + (1,)), np.zeros(ext + (3,)),
                                               sgrid.copy(), mom.copy())
    assert oracle.g2p2g(om, pts, order, [(1, 1.0, r_vel, r_mom), (0, -0.5, r_s, r_sg)],
                        [(0, 1.0, mass, r_mass), (1, 0.7, r_vel, r_mom2), (0, -0.5, r_s, r_sg)]) == 0
    tp = torch.tensor(pts, device="cuda")
    vel = torch.tensor(vel0, device="cuda").float()
    s = torch.tensor(s0[:, 0], device="cuda").float()
    tmass = torch.tensor(mass[:, 0], device="cuda").float()
    til = G.Tiling(mp, order, (8, 8, 8))
    perm = til.sort(tp, n)
    core.permute_by(perm, tp, vel, s, tmass)
    perm = perm.cpu().numpy()
    lay = lambda d: G.createArrayLayout(lg, d, M.Node)  # noqa: E731
    a_mom = G.createArray("mom", lay(3), torch.float32)
    a_mom.view().copy_(torch.tensor(mom, device="cuda").float())
    a_s = G.createArray("s", lay(1), torch.float32)
    a_s.view().copy_(torch.tensor(sgrid, device="cuda").float())
    a_mass, a_mom2 = G.createArray("m", lay(1), torch.float32), G.createArray("p", lay(3), torch.float32)
    G.g2p2g([G.createScalarValueP2G(tmass, 1.0), G.createVectorValueP2G(vel, 0.7), G.createScalarValueP2G(s, -0.5)],
            tp, n, G.Spline(order), G.createHalo(G.NodeHaloPattern(), 2), [a_mass, a_mom2, a_s],
            [G.createVectorValueG2P(vel, 1.0), G.createScalarValueG2P(s, -0.5)], [a_mom, a_s],
            precision=G.FP32_COMPENSATED, tiling=til, check_bounds=True)
    assert G.last_dispatch() == "tiled"
    assert max_rel(vel.double().cpu().numpy(), r_vel[perm]) <= 4e-6
    assert max_rel(s.double().cpu().numpy(), r_s[perm, 0]) <= 4e-6
    for got, ref in [(a_mass, r_mass), (a_mom2, r_mom2), (a_s, r_sg)]:
        assert max_rel(got.view().double().cpu().numpy(), ref) <= 2e-6, order
