"""Differentiable SC and Compton projectors for gradient-driven (MAP) reconstruction.

SCProject(x) = [A rot_r(x)]_r and ComptonProject(x) = T x (T recomputed from the event
records, never stored) are torch.autograd.Functions whose backward is the library's own
backprojector (jscc_sc_backproject / jscc_compton_backproject: the exact adjoints, same kernels
as the OSEM weights). The Poisson log-likelihood of the joint data,

    L(x) = sum_b (y_b log f_b - f_b) + sum_i log g_i - s_C . x,   f = A x,  g = T x,

has the gradient A^T(y / f) - A^T 1 + T^T(1 / g) - s_C, i.e. the OSEM weights minus the
sensitivities (recon_osem_plane.py:28-42), which tests/test_autograd_gpu.py checks.

RDPPrior is the relative-difference prior (jscc_rdp_prior: value and gradient in one pass,
the gradient kept for backward), and map_reconstruct minimises
-L(exp z) + beta R(exp z) over the log-parameterised image z.
"""
from __future__ import annotations

import torch

from . import ops


class SCProject(torch.autograd.Function):
    """f[b, r] = A[b] . rot_r(x) for r < n_rot; backward: sum_r rotinv_r(A^T g[:, r])."""

    @staticmethod
    def forward(ctx, x, sysmat, rotmat=None, rotmat_inv=None, n_rot=None, row_idx=None):
        ctx.sysmat, ctx.rotmat_inv, ctx.n_rot, ctx.row_idx = sysmat, rotmat_inv, n_rot, row_idx
        ctx.shape = x.shape
        return ops.sc_project(sysmat, x.detach(), rotmat=rotmat, n_rot=n_rot, row_idx=row_idx)

    @staticmethod
    def backward(ctx, g):
        grad = ops.sc_backproject(ctx.sysmat, g.contiguous(), rotmat_inv=ctx.rotmat_inv, n_rot=ctx.n_rot,
                                  row_idx=ctx.row_idx)
        return grad.reshape(ctx.shape), None, None, None, None, None


class ComptonProject(torch.autograd.Function):
    """g[i] = sum_j t_ij x_j over ComptonEvents (T recomputed); backward: T^T grad."""

    @staticmethod
    def forward(ctx, x, events, coor, sysmat, use_window=False):
        ctx.args = (events, coor, sysmat, use_window)
        ctx.shape = x.shape
        return ops.compton_project(events.records, events.row_id, coor, x.detach(), model=events.model, eff=sysmat,
                                   use_window=use_window)

    @staticmethod
    def backward(ctx, g):
        events, coor, sysmat, use_window = ctx.args
        grad = ops.compton_backproject(events.records, events.row_id, coor, g.contiguous(), model=events.model,
                                       eff=sysmat, use_window=use_window)
        return grad.reshape(ctx.shape), None, None, None, None


def sc_project(x, sysmat, rotmat=None, rotmat_inv=None, n_rot=None, row_idx=None):
    return SCProject.apply(x, sysmat, rotmat, rotmat_inv, n_rot, row_idx)


def compton_project(x, events, coor, sysmat, use_window=False):
    return ComptonProject.apply(x, events, coor, sysmat, use_window)


def poisson_log_likelihood(x, sc=None, compton=None, eps=float(torch.finfo(torch.float32).tiny)):
    """L(x) of the joint data. ``sc = (sysmat, proj [B, R], rotmat, rotmat_inv)`` (rotation
    tables may be None, then R = 1); ``compton = (events, coor, sysmat, s_c)`` with s_c the
    Compton sensitivity [V, 1] (the list-mode term's expected-count part). Differentiable in x.

    The projections come from the float32 kernels; the logarithms and the sums are taken in
    float64 (a float32 sum of ~1e4 terms carries a rounding error far above what a finite
    difference of L resolves). ``eps`` only keeps log() finite at exactly-zero projections:
    Compton projections of one event are routinely below 1e-12 and the OSEM weights use 1/f
    unclamped, so a larger floor would cut those events out of the gradient."""
    total = x.new_zeros((), dtype=torch.float64)
    if sc is not None:
        A, y, rot, rot_inv = sc
        n_rot = 1 if rot is None else y.reshape(y.size(0), -1).size(1)
        f = sc_project(x, A, rot, rot_inv, n_rot).double()
        yy = y.reshape(f.shape).double()
        total = total + (yy * torch.log(f.clamp_min(eps)) - f).sum()
    if compton is not None:
        events, coor, sysmat, s_c = compton
        g = compton_project(x, events, coor, sysmat).double()
        total = total + torch.log(g.clamp_min(eps)).sum() - (s_c.reshape(-1).double() * x.reshape(-1).double()).sum()
    return total


class RDPPrior(torch.autograd.Function):
    """beta R(x) over a NeighbourTable; the forward pass computes the gradient too."""

    @staticmethod
    def forward(ctx, x, table, beta, gamma, eps):
        value, grad = ops.rdp_prior(x.detach(), table.nbr, table.weight, gamma=gamma, beta=beta, eps=eps)
        ctx.save_for_backward(grad)
        ctx.shape = x.shape
        return value

    @staticmethod
    def backward(ctx, gv):
        (grad,) = ctx.saved_tensors
        return (grad * gv.to(grad.dtype)).reshape(ctx.shape), None, None, None, None


def rdp_prior(x, table, beta=0.01, gamma=2.0, eps=1e-9):
    """beta R(x) (float64 0-d tensor), differentiable in x."""
    return RDPPrior.apply(x, table, beta, gamma, eps)


def map_reconstruct(x0, sc=None, compton=None, table=None, beta=0.01, gamma=2.0, n_steps=200, lr=0.05,
                    eps=1e-9, callback=None):
    """MAP estimate on a log-parameterised image: minimise
    Phi(z) = -L(exp z) + beta R(exp z) with Adam (``lr`` is a step in log-intensity, so it is
    scale-free). ``sc`` / ``compton`` as in poisson_log_likelihood; ``table`` a NeighbourTable
    on the device (None: no prior). Returns (x, objective history [n_steps] float64 on the
    host); ``callback(step, x, objective)`` is called after each step with device tensors."""
    z = torch.log(x0.detach().float().clamp_min(torch.finfo(torch.float32).tiny)).requires_grad_(True)
    opt = torch.optim.Adam([z], lr=lr)
    hist = []
    for it in range(n_steps):
        opt.zero_grad(set_to_none=False)
        x = torch.exp(z)
        obj = -poisson_log_likelihood(x, sc=sc, compton=compton)
        if table is not None and beta != 0:
            obj = obj + rdp_prior(x, table, beta=beta, gamma=gamma, eps=eps)
        obj.backward()
        opt.step()
        hist.append(obj.detach())
        if callback is not None:
            callback(it, torch.exp(z.detach()), obj.detach())
    return torch.exp(z.detach()), torch.stack(hist).cpu() if hist else torch.zeros(0, dtype=torch.float64)
