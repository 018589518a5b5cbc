"""Differentiable filter -> interpolation chain.

``FilterInterp.apply(x, filt, interp)`` returns P F x for a design field x
(node-major, ``vpn`` components per filter node): the matrix density filter
F on the filter forest followed by the prolongation P to a finer forest.
The backward pass is the exact adjoint F^T P^T, computed by the library's
transpose kernels (no recomputation, nothing saved but the operators).
"""
import torch

from .TMR import MatrixFilter, VecInterp


class FilterInterp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, filt: MatrixFilter, interp: VecInterp, vpn: int = 1):
        if x.dtype != torch.float64:
            raise TypeError("FilterInterp: the interpolation apply is FP64")
        x = x.contiguous()
        rows, cols, _ = interp.sizes()
        n = filt.size()[0]
        if n != cols:
            raise ValueError("FilterInterp: filter has %d nodes, P has %d columns" % (n, cols))
        if x.numel() != n * vpn:
            raise ValueError("FilterInterp: x holds %d values, expected %d nodes x vpn %d"
                             % (x.numel(), n, vpn))
        rho_f = torch.empty_like(x)
        filt.applyFilter(x, rho_f, vpn)
        y = torch.empty(rows * vpn, dtype=x.dtype, device=x.device)
        interp.mult(rho_f, y)
        ctx.filt, ctx.interp, ctx.vpn = filt, interp, vpn
        ctx.ncols = cols
        return y

    @staticmethod
    def backward(ctx, gy):
        gy = gy.contiguous()
        g = torch.empty(ctx.ncols * ctx.vpn, dtype=gy.dtype, device=gy.device)
        ctx.interp.multTranspose(gy, g)
        gx = torch.empty_like(g)
        ctx.filt.applyTranspose(g, gx, ctx.vpn)
        return gx, None, None, None


def filter_interp(x, filt, interp, vpn=1):
    return FilterInterp.apply(x, filt, interp, vpn)
