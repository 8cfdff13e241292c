"""Batched launches (cgx_batch_*): many independent meshes, one work list,
one persistent kernel per direction.

* Per instance the batched P2G / G2P equal the single-instance tiled calls
  (same kernels; only the order of float atomics differs: 1e-6) and the FP64
  oracle (grid 1e-6, point fields 2e-6).
* A plan executed inside a CUDA graph gives the eager results.
* The autotuner picks a setting from its candidates and the results are
  unchanged under it.
* Periodic instances run their halo step inside the batch.
"""
import numpy as np
import pytest
import torch

from cabana_gb300 import grid as G
from cabana_gb300 import mesh as M
from tests.helpers import clumped_points, domain, max_rel, oracle_mesh

pytestmark = pytest.mark.gpu

ORDER = 2


def _make_batch(n_inst, seed, side=(16, 40), parts=(1e3, 1e5), periodic_every=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_inst):
        n_side = int(rng.integers(side[0], side[1] + 1))
        periodic = periodic_every > 0 and i % periodic_every == 0
        lg, mp = M.simple_mesh(n_side, 0.5, tuple(rng.uniform(-2, 2, 3)), 1, periodic=(periodic,) * 3)
        lo, hi = domain(mp)
        npart = int(np.exp(rng.uniform(np.log(parts[0]), np.log(parts[1]))))
        clumps = int(rng.integers(0, 9))
        pts = (rng.uniform(lo, hi, size=(npart, 3)) if clumps == 0
               else clumped_points(rng, npart, lo, hi, clumps, 1.5))
        pos = torch.tensor(pts, device="cuda")
        mass = torch.tensor(rng.uniform(0.5, 1.5, npart), dtype=torch.float32, device="cuda")
        vel = torch.tensor(rng.normal(size=(npart, 3)), dtype=torch.float32, device="cuda")
        til = G.Tiling(mp, ORDER, (8, 8, 8))
        perm = til.sort(pos, npart)
        pos, mass, vel = pos[perm].contiguous(), mass[perm].contiguous(), vel[perm].contiguous()
        mom = (mass[:, None] * vel).contiguous()
        out.append(dict(lg=lg, mp=mp, pos=pos, mass=mass, mom=mom, n=npart, til=til,
                        mass_g=G.createArray("m", G.createArrayLayout(lg, 1, G.Node), torch.float32),
                        mom_g=G.createArray("p", G.createArrayLayout(lg, 3, G.Node), torch.float32),
                        v=torch.zeros(npart, 3, device="cuda"), vg=torch.zeros(npart, 3, 3, device="cuda")))
    return out


def _plans(batch):
    p2g = [G.createScalarValueP2G(None, 1.0), G.createVectorValueP2G(None, 1.0)]
    g2p = [G.createVectorValueG2P(None, 1.0), G.createVectorGradientG2P(None, 1.0)]
    pi = [G.BatchInstance(b["pos"], b["n"], b["til"], [b["mass"], b["mom"]], [b["mass_g"], b["mom_g"]]) for b in batch]
    gi = [G.BatchInstance(b["pos"], b["n"], b["til"], [b["v"], b["vg"]], [b["mom_g"], b["mom_g"]]) for b in batch]
    return G.BatchPlan(p2g, pi, G.Spline(ORDER), p2g=True), G.BatchPlan(g2p, gi, G.Spline(ORDER), p2g=False)


def _zero(batch):
    for b in batch:
        b["mass_g"].view().zero_()
        b["mom_g"].view().zero_()
        b["v"].zero_()
        b["vg"].zero_()


def _snapshot(batch):
    return [tuple(t.clone() for t in (b["mass_g"].view(), b["mom_g"].view(), b["v"], b["vg"])) for b in batch]


def _single(b):
    """Per-instance tiled calls: the per-instance-launch form of the same work."""
    halo = G.createHalo(G.NodeHaloPattern(), 1)
    mg = G.createArray("m", G.createArrayLayout(b["lg"], 1, G.Node), torch.float32)
    pg = G.createArray("p", G.createArrayLayout(b["lg"], 3, G.Node), torch.float32)
    G.p2g([G.createScalarValueP2G(b["mass"], 1.0), G.createVectorValueP2G(b["mom"], 1.0)], b["pos"], b["n"],
          G.Spline(ORDER), halo, [mg, pg], precision=G.FP32_COMPENSATED, tiling=b["til"])
    v = torch.zeros(b["n"], 3, device="cuda")
    vg = torch.zeros(b["n"], 3, 3, device="cuda")
    G.g2p(pg, halo, b["pos"], b["n"], G.Spline(ORDER), [G.createVectorValueG2P(v, 1.0),
                                                         G.createVectorGradientG2P(vg, 1.0)],
          precision=G.FP32_COMPENSATED, tiling=b["til"])
    return mg.view(), pg.view(), v, vg


def _check_against_single(batch, snap, tol=1e-6):
    for b, got in zip(batch, snap):
        ref = _single(b)
        for g, r in zip(got, ref):
            assert max_rel(g.double().cpu().numpy(), r.double().cpu().numpy()) <= tol


def test_batch_matches_single_instance_calls():
    batch = _make_batch(40, 1, periodic_every=7)
    pp, gp = _plans(batch)
    _zero(batch)
    pp.execute()
    gp.execute()
    torch.cuda.synchronize()
    _check_against_single(batch, _snapshot(batch))


def test_batch_matches_oracle(oracle):
    batch = _make_batch(6, 2, periodic_every=3)
    pp, gp = _plans(batch)
    _zero(batch)
    pp.execute()
    gp.execute()
    torch.cuda.synchronize()
    for b in batch:
        om = oracle_mesh(oracle, b["mp"])
        pts = b["pos"].cpu().numpy()
        ext = b["mp"].extents()
        mg = np.zeros(ext + (1,))
        pg = np.zeros(ext + (3,))
        oracle.p2g(om, pts, ORDER, [(0, 1.0, b["mass"].double().cpu().numpy().reshape(-1, 1).copy(), mg),
                                    (1, 1.0, b["mom"].double().cpu().numpy().copy(), pg)])
        oracle.halo_gather(om, pg)  # the batched g2p gathered the momentum array in place
        assert max_rel(b["mass_g"].view().double().cpu().numpy(), mg) <= 1e-6
        assert max_rel(b["mom_g"].view().double().cpu().numpy(), pg) <= 1e-6
        # g2p reads the FP32 grid the batch produced
        pg32 = b["mom_g"].view().double().cpu().numpy().copy()
        v = np.zeros((b["n"], 3))
        vg = np.zeros((b["n"], 9))
        oracle.g2p(om, pts, ORDER, [(1, 1.0, v, pg32), (3, 1.0, vg, pg32)])
        assert max_rel(b["v"].double().cpu().numpy(), v) <= 2e-6
        assert max_rel(b["vg"].double().cpu().numpy().reshape(-1, 9), vg) <= 2e-6


def test_batch_in_cuda_graph():
    batch = _make_batch(30, 3)
    pp, gp = _plans(batch)
    _zero(batch)
    pp.execute()
    gp.execute()
    torch.cuda.synchronize()
    eager = _snapshot(batch)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            _zero(batch)
            pp.execute(stream=s)
            gp.execute(stream=s)
    for _ in range(2):
        graph.replay()
    torch.cuda.synchronize()
    for e, g in zip(eager, _snapshot(batch)):
        for a, b in zip(e, g):
            assert max_rel(b.double().cpu().numpy(), a.double().cpu().numpy()) <= 1e-6


def test_batch_autotune():
    batch = _make_batch(30, 4)
    pp, gp = _plans(batch)
    for plan in (pp, gp):
        best = plan.autotune()
        assert best > 0.0
        item, ctas = plan.config()
        assert item in (1024, 2048, 4096, 8192, 16384) and ctas >= 1
    pp.set_config(512, 1)
    assert pp.config() == (512, 1)
    _zero(batch)
    pp.execute()
    gp.execute()
    torch.cuda.synchronize()
    _check_against_single(batch, _snapshot(batch))
