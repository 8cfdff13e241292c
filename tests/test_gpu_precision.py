"""Large-origin precision sweep (FP32-compensated form against the plain FP64
form, which is itself within 1e-12 of the FP64 oracle in
test_gpu_interpolation.py).

128^3 cells whose low corner sits at 1e6 cell widths in every dimension;
16,777,216 uniform particles plus 1,677,722 (10 %) in one Gaussian clump of
sigma 4 cells; Spline<1>, <2>, <3>. P2G ScalarValue(mass),
VectorValue(momentum), ScalarGradient(mass); G2P ScalarGradient of the mass
grid. Bars: grid max-relative error <= 1e-6 (gradient channel: 2e-6 against
its largest entry, 1e-6 in L2), point field <= 4e-6 (the
gradient of a nearly uniform mass field, relative to its largest value: FP32
cancellation in the gather), mass and
momentum conservation <= 1e-6 (sums formed in FP64).
"""
import pytest
import torch

from cabana_gb300 import grid as G
from cabana_gb300 import mesh as M

pytestmark = pytest.mark.gpu

CELLS = 128
OFFSET = 1.0e6


def _points(seed):
    gen = torch.Generator(device="cuda").manual_seed(seed)
    lo = OFFSET
    n_uni, n_clump = 1 << 24, 1677722
    uni = lo + torch.rand(n_uni, 3, device="cuda", dtype=torch.float64, generator=gen) * CELLS
    centre = lo + torch.rand(1, 3, device="cuda", dtype=torch.float64, generator=gen) * CELLS
    clump = centre + torch.randn(n_clump, 3, device="cuda", dtype=torch.float64, generator=gen) * 4.0
    for _ in range(64):
        bad = ((clump < lo) | (clump >= lo + CELLS)).any(dim=1)
        nb = int(bad.sum())
        if nb == 0:
            break
        clump[bad] = centre + torch.randn(nb, 3, device="cuda", dtype=torch.float64, generator=gen) * 4.0
    pos = torch.cat([uni, clump])
    mass = torch.rand(pos.shape[0], device="cuda", generator=gen) + 0.5
    vel = torch.randn(pos.shape[0], 3, device="cuda", generator=gen)
    return pos, mass, (mass[:, None] * vel).contiguous()


def _run(lg, pos, n, order, mass, mom, dtype, precision, tiling):
    arrs = [G.createArray(l, G.createArrayLayout(lg, d, G.Node), dtype) for l, d in (("m", 1), ("p", 3), ("g", 3))]
    G.p2g([G.createScalarValueP2G(mass, 1.0), G.createVectorValueP2G(mom, 1.0), G.createScalarGradientP2G(mass, 1.0)],
          pos, n, G.Spline(order), None, arrs, precision=precision, tiling=tiling)
    grad = torch.zeros(n, 3, dtype=dtype, device="cuda")
    G.g2p(arrs[0], None, pos, n, G.Spline(order), G.createScalarGradientG2P(grad, 1.0), precision=precision,
          tiling=tiling)
    return [a.view() for a in arrs], grad


def _mrel(a, b):
    return float((a.double() - b.double()).abs().max() / b.double().abs().max())


@pytest.mark.parametrize("order", [1, 2, 3])
def test_large_origin_precision(order):
    lg, mp = M.simple_mesh(CELLS, 1.0, (OFFSET,) * 3, 1)
    pos, mass, mom = _points(3)
    n = pos.shape[0]
    til = G.Tiling(mp, order, (8, 8, 8))
    perm = til.sort(pos, n)
    pos, mass, mom = pos[perm].contiguous(), mass[perm].contiguous(), mom[perm].contiguous()
    (m32, p32, g32), gr32 = _run(lg, pos, n, order, mass, mom, torch.float32, G.FP32_COMPENSATED, til)
    assert G.last_dispatch() == "tiled"
    (m64, p64, g64), gr64 = _run(lg, pos, n, order, mass.double(), mom.double(), torch.float64, G.PLAIN_FP64, None)
    assert _mrel(m32, m64) <= 1e-6
    assert _mrel(p32, p64) <= 1e-6
    # the gradient channel sums terms of both signs; measured against its
    # largest entry it carries the FP32 rounding of every term (~1e-6 for the
    # cubic spline), in the L2 norm it stays well inside 1e-6
    assert _mrel(g32, g64) <= 2e-6
    assert float((g32.double() - g64).norm() / g64.norm()) <= 1e-6
    assert _mrel(gr32, gr64) <= 4e-6
    msum = mass.double().sum()
    assert abs(float(m32.double().sum() - msum) / float(msum)) <= 1e-6
    psum = mom.double().sum(dim=0)
    assert float((p32.double().sum(dim=(0, 1, 2)) - psum).abs().max() / mom.double().abs().sum(dim=0).max()) <= 1e-6


def test_cpu_reference_case(oracle):
    """The reference's CPU-runnable case: 32^3 cells of size 1 from the
    origin, one halo cell, non-periodic (35^3 ghosted nodes), 262,144
    particles uniform in [0, 32)^3, mass U(0.5, 1.5), velocity N(0, 1)^3,
    momentum = m v in FP64, Spline<3>; ScalarValueP2G(mass) +
    VectorValueP2G(momentum), then VectorValueG2P(velocity) from the momentum
    grid. Seed 0. Plain FP64 within 1e-12 of the oracle, the FP32 tiled form
    within 1e-6 (grid) / 2e-6 (points)."""
    import numpy as np
    from tests.helpers import max_rel, oracle_mesh
    rng = np.random.default_rng(0)
    n = 262144
    pts = rng.uniform(0.0, 32.0, size=(n, 3))
    mass = rng.uniform(0.5, 1.5, n)
    vel = rng.normal(size=(n, 3))
    mom = mass[:, None] * vel
    lg, mp = M.simple_mesh(32, 1.0, (0.0, 0.0, 0.0), 1)
    om = oracle_mesh(oracle, mp)
    ext = mp.extents()
    assert ext == (35, 35, 35)
    mg = np.zeros(ext + (1,))
    pg = np.zeros(ext + (3,))
    oracle.p2g(om, pts, 3, [(0, 1.0, mass.reshape(-1, 1).copy(), mg), (1, 1.0, mom.copy(), pg)])
    v_ref = np.zeros((n, 3))
    oracle.g2p(om, pts, 3, [(1, 1.0, v_ref, pg.copy())])
    # plain FP64
    pos = torch.tensor(pts, device="cuda")
    arrs = [G.createArray("m", G.createArrayLayout(lg, 1, G.Node), torch.float64),
            G.createArray("p", G.createArrayLayout(lg, 3, G.Node), torch.float64)]
    G.p2g([G.createScalarValueP2G(torch.tensor(mass, device="cuda"), 1.0),
           G.createVectorValueP2G(torch.tensor(mom, device="cuda"), 1.0)], pos, n, G.Spline(3),
          G.createHalo(G.NodeHaloPattern(), 1), arrs)
    v = torch.zeros(n, 3, dtype=torch.float64, device="cuda")
    G.g2p(arrs[1], G.createHalo(G.NodeHaloPattern(), 1), pos, n, G.Spline(3), G.createVectorValueG2P(v, 1.0))
    assert max_rel(arrs[0].view().cpu().numpy(), mg) <= 1e-12
    assert max_rel(arrs[1].view().cpu().numpy(), pg) <= 1e-12
    assert max_rel(v.cpu().numpy(), v_ref) <= 1e-12
    # FP32 tiled, on the tile-sorted copy
    til = G.Tiling(mp, 3, (8, 8, 8))
    perm = til.sort(pos, n)
    p_np = perm.cpu().numpy()
    pos_s = pos[perm].contiguous()
    a32 = [G.createArray("m", G.createArrayLayout(lg, 1, G.Node), torch.float32),
           G.createArray("p", G.createArrayLayout(lg, 3, G.Node), torch.float32)]
    G.p2g([G.createScalarValueP2G(torch.tensor(mass[p_np], dtype=torch.float32, device="cuda"), 1.0),
           G.createVectorValueP2G(torch.tensor(mom[p_np], dtype=torch.float32, device="cuda"), 1.0)], pos_s, n,
          G.Spline(3), None, a32, precision=G.FP32_COMPENSATED, tiling=til)
    assert G.last_dispatch() == "tiled"
    v32 = torch.zeros(n, 3, device="cuda")
    G.g2p(a32[1], None, pos_s, n, G.Spline(3), G.createVectorValueG2P(v32, 1.0), precision=G.FP32_COMPENSATED,
          tiling=til)
    assert max_rel(a32[0].view().double().cpu().numpy(), mg) <= 1e-6
    assert max_rel(a32[1].view().double().cpu().numpy(), pg) <= 1e-6
    assert max_rel(v32.double().cpu().numpy(), v_ref[p_np]) <= 2e-6
