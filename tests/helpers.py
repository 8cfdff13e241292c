"""Shared helpers for the parity tests: seeded inputs, oracle runs, error
metrics. The oracle (oracle/oracle.py) is the checker; the GPU side goes
through cabana_gb300 (libcgx.so) only."""
import numpy as np

from cabana_gb300 import mesh as M

# kind 5: the transposed tensor operators (no reference counterpart; adjoints)
P2G_COMPS = {0: 1, 1: 3, 2: 1, 3: 3, 4: 9, 5: 9}
P2G_DOFS = {0: 1, 1: 3, 2: 3, 3: 1, 4: 3, 5: 3}
G2P_COMPS = {0: 1, 1: 3, 2: 3, 3: 9, 4: 1, 5: 9}
G2P_DOFS = {0: 1, 1: 3, 2: 1, 3: 3, 4: 3, 5: 3}
P2G_NAMES = ["ScalarValueP2G", "VectorValueP2G", "ScalarGradientP2G", "VectorDivergenceP2G", "TensorDivergenceP2G"]
G2P_NAMES = ["ScalarValueG2P", "VectorValueG2P", "ScalarGradientG2P", "VectorGradientG2P", "VectorDivergenceG2P"]


def oracle_mesh(oracle, mp):
    return oracle.make_mesh(mp.ghost_low, mp.cell_size, mp.owned_cells, mp.halo_width, mp.periodic, mp.entity)


def uniform_points(rng, n, lo, hi):
    return rng.uniform(lo, hi, size=(n, 3))


def clumped_points(rng, n, lo, hi, clumps, sigma):
    """Gaussian clumps with centres uniform in [lo, hi); draws outside the box
    are redrawn from the same clump."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    centres = rng.uniform(lo, hi, size=(clumps, 3))
    which = rng.integers(0, clumps, size=n)
    pts = centres[which] + rng.normal(0.0, sigma, size=(n, 3))
    bad = np.any((pts < lo) | (pts >= hi), axis=1)
    while bad.any():
        k = int(bad.sum())
        pts[bad] = centres[which[bad]] + rng.normal(0.0, sigma, size=(k, 3))
        bad = np.any((pts < lo) | (pts >= hi), axis=1)
    return pts


def domain(mp):
    """Owned physical box [lo, hi) of a mesh."""
    lo = tuple(mp.ghost_low[d] + mp.halo_width * mp.cell_size[d] for d in range(3))
    hi = tuple(lo[d] + mp.owned_cells[d] * mp.cell_size[d] for d in range(3))
    return lo, hi


def max_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.max(np.abs(b))
    if den == 0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / den)


def l2_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b.ravel())
    if den == 0:
        return float(np.linalg.norm(a.ravel()))
    return float(np.linalg.norm((a - b).ravel()) / den)
