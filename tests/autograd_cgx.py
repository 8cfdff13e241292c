"""Test-only torch.autograd.Functions over libcgx's forward and adjoint calls.

P2GMomentum: grid = VectorValueP2G(momentum) at the points (plus an optional
TensorDivergenceP2G of a stress); backward = cgx_p2g_adjoint.
G2PVelocity: velocity = VectorValueG2P(grid) at the points; backward =
cgx_g2p_adjoint. Positions are differentiable in both. These wrap the C ABI
through cabana_gb300.grid only; nothing here computes on its own.
"""
import torch

from cabana_gb300 import grid as G


class _Ctx:
    def __init__(self, local_grid, order, precision, tiling=None, halo=True):
        self.lg = local_grid
        self.order = order
        self.precision = precision
        self.tiling = tiling
        self.halo = G.createHalo(G.NodeHaloPattern(), 1) if halo else None


def _array(ctx, dofs, dtype, data=None):
    a = G.createArray("a", G.createArrayLayout(ctx.lg, dofs, G.Node), dtype)
    if data is not None:
        a.view().copy_(data)
    return a


class P2GMomentum(torch.autograd.Function):
    @staticmethod
    def forward(fctx, pos, mom, ctx, mult):
        arr = _array(ctx, 3, mom.dtype)
        f = G.createVectorValueP2G(mom.detach().contiguous(), mult)
        G.p2g(f, pos.detach().contiguous(), pos.shape[0], G.Spline(ctx.order), ctx.halo, arr,
              precision=ctx.precision, tiling=ctx.tiling)
        fctx.save_for_backward(pos, mom)
        fctx.cgx = (ctx, mult)
        return arr.view().clone()

    @staticmethod
    def backward(fctx, grid_bar):
        pos, mom = fctx.saved_tensors
        ctx, mult = fctx.cgx
        gbar = _array(ctx, 3, mom.dtype, grid_bar)
        mom_bar = torch.zeros_like(mom)
        pos_bar = torch.zeros_like(pos)
        f = G.createVectorValueP2G(mom.detach().contiguous(), mult)
        G.p2g_adjoint(f, pos.detach().contiguous(), pos.shape[0], G.Spline(ctx.order), ctx.halo, gbar,
                      x_bar=mom_bar, points_bar=pos_bar, precision=ctx.precision, tiling=ctx.tiling)
        return pos_bar, mom_bar, None, None


class G2PVelocity(torch.autograd.Function):
    @staticmethod
    def forward(fctx, pos, grid, ctx, mult):
        arr = _array(ctx, 3, grid.dtype, grid)
        vel = torch.zeros(pos.shape[0], 3, dtype=grid.dtype, device=grid.device)
        f = G.createVectorValueG2P(vel, mult)
        G.g2p(arr, ctx.halo, pos.detach().contiguous(), pos.shape[0], G.Spline(ctx.order), f,
              precision=ctx.precision, tiling=ctx.tiling)
        fctx.save_for_backward(pos, arr.view().clone())  # the array as the forward read it
        fctx.cgx = (ctx, mult)
        return vel

    @staticmethod
    def backward(fctx, vel_bar):
        pos, read = fctx.saved_tensors
        ctx, mult = fctx.cgx
        arr = _array(ctx, 3, read.dtype, read)
        gbar = _array(ctx, 3, read.dtype)
        pos_bar = torch.zeros_like(pos)
        f = G.createVectorValueG2P(torch.zeros(pos.shape[0], 3, dtype=read.dtype, device=read.device), mult)
        G.g2p_adjoint(arr, ctx.halo, pos.detach().contiguous(), pos.shape[0], G.Spline(ctx.order), f,
                      vel_bar.contiguous(), array_bar=gbar, points_bar=pos_bar, precision=ctx.precision,
                      tiling=ctx.tiling)
        return pos_bar, gbar.view().clone(), None, None
