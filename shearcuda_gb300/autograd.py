"""Differentiable NSST denoising: torch.autograd over the hand-written adjoint.

loss = f(NSST^-1(T(NSST(x), tau))) with per-band thresholds tau (one per
band, shared by the images of a batch).  Forward and backward both run in
libnsst.so (nsst_denoise_tau_batch / nsst_denoise_tau_backward); PyTorch only
routes gradients.  Batches larger than the plan's capacity are processed in
chunks.  When the whole batch fits the plan and nothing else ran on the plan
since the forward, the backward reuses the band coefficients the forward left
in the plan (nsst_denoise_tau_backward_saved); otherwise it recomputes them
chunk by chunk, so memory does not grow with the batch.
"""
import ctypes

import numpy as np
import torch

from ._lib import NsstError, THRESH_SOFT, check, lib
from .ops import ShearPlan, _stream

__all__ = ['NsstDenoiseFn', 'nsst_denoise_diff', 'NsstDenoiser', 'shear_trans_adjoint', 'inverse_shear_adjoint']


def _ptrs(t, n):
    base = t.data_ptr()
    step = t[0].numel() * t.element_size()
    return (ctypes.c_void_p * n)(*[base + i * step for i in range(n)])


def _check_stack(x, plan, name):
    if not (x.is_cuda and x.dtype == torch.float32 and x.dim() == 3 and tuple(x.shape[1:]) == (plan.H, plan.W)):
        raise NsstError(1, '%s must be a CUDA float32 tensor of shape (n, %d, %d)' % (name, plan.H, plan.W))


class NsstDenoiseFn(torch.autograd.Function):
    """out = R(T(A x, tau)) for x of shape (n, H, W) and tau of shape (nbands,)."""

    @staticmethod
    def forward(ctx, x, tau, plan, mode):
        _check_stack(x, plan, 'x')
        x = x.contiguous()
        tau = tau.contiguous()
        if tau.numel() != plan.nbands or not tau.is_cuda or tau.dtype != torch.float32:
            raise NsstError(1, 'tau must be a CUDA float32 tensor with %d entries' % plan.nbands)
        out = torch.empty_like(x)
        st = _stream()
        for c0 in range(0, x.shape[0], plan.batch):
            xs, os_ = x[c0:c0 + plan.batch], out[c0:c0 + plan.batch]
            n = xs.shape[0]
            check(lib().nsst_denoise_tau_batch(plan.handle, _ptrs(xs, n), _ptrs(os_, n), n,
                                               ctypes.c_void_p(tau.data_ptr()), mode, st))
        plan._diff_token = getattr(plan, '_diff_token', 0) + 1
        ctx.save_for_backward(x, tau)
        ctx.plan, ctx.mode, ctx.token = plan, mode, plan._diff_token
        ctx.single = x.shape[0] <= plan.batch
        return out

    @staticmethod
    def backward(ctx, grad_out):
        x, tau = ctx.saved_tensors
        plan, mode = ctx.plan, ctx.mode
        grad_out = grad_out.contiguous()
        gx = torch.empty_like(x)
        gtau = torch.zeros_like(tau)
        st = _stream()
        n = x.shape[0]
        if (ctx.single and ctx.token == getattr(plan, '_diff_token', -1)
                and lib().nsst_plan_saved_items(plan.handle) == n):
            check(lib().nsst_denoise_tau_backward_saved(plan.handle, _ptrs(grad_out, n), _ptrs(gx, n), n,
                                                        ctypes.c_void_p(tau.data_ptr()),
                                                        ctypes.c_void_p(gtau.data_ptr()), 0, mode, st))
            return gx, gtau, None, None
        for k, c0 in enumerate(range(0, x.shape[0], plan.batch)):
            xs, gs, gxs = x[c0:c0 + plan.batch], grad_out[c0:c0 + plan.batch], gx[c0:c0 + plan.batch]
            n = xs.shape[0]
            check(lib().nsst_denoise_tau_backward(plan.handle, _ptrs(xs, n), _ptrs(gs, n), _ptrs(gxs, n), n,
                                                  ctypes.c_void_p(tau.data_ptr()), ctypes.c_void_p(gtau.data_ptr()),
                                                  1 if k > 0 else 0, mode, st))
        return gx, gtau, None, None


def nsst_denoise_diff(x, tau, plan, mode=THRESH_SOFT):
    """Differentiable batched denoise; x (n, H, W) or (H, W)."""
    squeeze = x.dim() == 2
    if squeeze:
        x = x.unsqueeze(0)
    out = NsstDenoiseFn.apply(x, tau, plan, mode)
    return out[0] if squeeze else out


class NsstDenoiser(torch.nn.Module):
    """Learnable per-band thresholds tau_b, initialised at k_level * sigma * scalar_b."""

    def __init__(self, plan, scalars, sigma, K, mode=THRESH_SOFT, device='cuda'):
        super().__init__()
        if plan.batch < 1:
            raise NsstError(1, 'bad plan')
        lib().nsst_plan_enable_grad(plan.handle)
        self.plan, self.mode = plan, mode
        K = np.asarray(K, np.float64)
        init = np.array([K[lv] * sigma * s for lv, s in zip(plan.band_levels, np.asarray(scalars, np.float64))])
        self.tau = torch.nn.Parameter(torch.tensor(init, dtype=torch.float32, device=device))

    def forward(self, x):
        return nsst_denoise_diff(x, self.tau, self.plan, self.mode)


def enable_grad(plan):
    check(lib().nsst_plan_enable_grad(plan.handle))


def shear_trans_adjoint(coeffs, plan, stream=None):
    """x = A^T c (adjoint of shear_trans_cuda)."""
    enable_grad(plan)
    x = torch.empty((plan.H, plan.W), device=coeffs.device, dtype=torch.float32)
    check(lib().nsst_shear_trans_adjoint(plan.handle, ctypes.c_void_p(coeffs.contiguous().data_ptr()),
                                         ctypes.c_void_p(x.data_ptr()), _stream(stream)))
    return x


def inverse_shear_adjoint(x, plan, stream=None):
    """c = R^T x (adjoint of inverse_shear_cuda)."""
    enable_grad(plan)
    c = torch.empty((plan.nbands, plan.H, plan.W), device=x.device, dtype=torch.float32)
    check(lib().nsst_inverse_shear_adjoint(plan.handle, ctypes.c_void_p(x.contiguous().data_ptr()),
                                           ctypes.c_void_p(c.data_ptr()), _stream(stream)))
    return c
