"""Python mirror of ShearCuda's 3-D operator surface (``shearcuda3d``) over libnsst.so.

=============================  ==========================================================================
here                           reference (ShearCuda tree)
=============================  ==========================================================================
``VolumePlan``                 GetMeyerBasedFilter.m:12-150 + the buffers ShDecThRec_cuda.cpp:178-335 makes
``get_meyer_based_filter``     shearcuda3d/3DShearTrans/GetMeyerBasedFilter.m:12-150 (FP64, host)
``do_pyr_dec``                 shearcuda3d/3DShearTrans/DoPyrDec.m:1-6 (PyrNDDec_mm.m:20-109, Pyr_mode 1.5)
``do_pyr_rec``                 shearcuda3d/3DShearTrans/DoPyrRec.m:1-4 (PyrNDRec_mm.m:20-95)
``sh_dec``                     shearcuda3d/3DShearTrans/ShDec.m:18-34 (convnfft 'same', one level)
``sh_dec_th_rec_cuda``         shearcuda3d/3DShearTrans/src_cuda/ShDecThRec_cuda.cpp:57-335
``nsst_scalars3``              shearcuda3d/DenoiseDemo/NsstScalars.m:1-19
``denoise3``                   shearcuda3d/DenoiseDemo/main.m:80-145 (fused, batched)
``denoise3_backward``          (no reference counterpart) adjoint of ``denoise3`` at its threshold masks
``Denoise3Fn``                 ``torch.autograd.Function`` over ``denoise3`` / ``denoise3_backward``
=============================  ==========================================================================

Volumes are CUDA float32 tensors (n0, n1, n2) or batches (B, n0, n1, n2);
axis k plays MATLAB dimension k+1.  Sub-bands come back as a list
``[bp level 0 (finest), ..., lowpass]`` of views into one flat tensor, the
``BP`` cell of DoPyrDec.m.
"""
import ctypes

import numpy as np
import torch

from ._lib import GRID_FAST, GRID_MARSHAL, Nsst3Config, NsstError, check, lib
from .ops import _dev, _dptr, _stream

__all__ = ['VolumePlan', 'get_meyer_based_filter', 'do_pyr_dec', 'do_pyr_rec', 'sh_dec', 'sh_dec_th_rec_cuda',
           'nsst_scalars3', 'denoise3', 'denoise3_backward', 'Denoise3Fn', 'denoise3_diff', 'DEMO_T',
           'DEMO_NUM_DIRS', 'V3_NUM_DIRS']

DEMO_T = (3.3, 3.0, 3.0, 3.0)     # DenoiseDemo/main.m:18
DEMO_NUM_DIRS = (8, 4, 4)         # dBand{3} of DenoiseDemo/main.m:44-47 (numDir per level, finest first)
V3_NUM_DIRS = (2, 2, 4)           # 4, 4 and 16 directions per cone per level: 72 bands


def get_meyer_based_filter(num_dirs):
    """FP64 Meyer filters, (nbands, 24, 24, 24) in band order (level, cone, l2, l1)."""
    nd = (ctypes.c_int * len(num_dirs))(*[int(v) for v in num_dirs])
    count = lib().nsst3_meyer_filters(len(num_dirs), nd, None)
    if count < 0:
        raise NsstError(1, 'num_dirs must divide 24 and lie in [2, 12]')
    out = np.empty((count, 24, 24, 24), dtype=np.float64)
    lib().nsst3_meyer_filters(len(num_dirs), nd, _dptr(out))
    return out


class VolumePlan:
    """Filters, windows and work buffers for batches of up to ``batch``
    volumes of size (n0, n1, n2)."""

    def __init__(self, n0, n1, n2, num_dirs=V3_NUM_DIRS, pyr_mode=1.5, batch=1, grid='fast'):
        """grid: 'fast' (edge replication to a 2^a 3^b grid) or 'marshal'
        (MarshalData.m's padding, as the reference's any-size demo)."""
        cfg = Nsst3Config()
        cfg.nlevels = len(num_dirs)
        for i, v in enumerate(num_dirs):
            cfg.num_dirs[i] = int(v)
        cfg.pyr_mode = float(pyr_mode)
        cfg.grid = {'fast': GRID_FAST, 'marshal': GRID_MARSHAL}[grid]
        h = ctypes.c_void_p()
        check(lib().nsst3_plan_create(ctypes.byref(cfg), int(n0), int(n1), int(n2), int(batch), ctypes.byref(h)))
        self._h = h
        self.shape = (int(n0), int(n1), int(n2))
        self.num_dirs = tuple(int(v) for v in num_dirs)
        self.nlevels = len(num_dirs)
        self.batch = int(batch)
        self.nbands = lib().nsst3_num_bands(h)
        self.subband_floats = lib().nsst3_subband_floats(h)
        d = (ctypes.c_int * 3)()
        c = (ctypes.c_int * 3)()
        check(lib().nsst3_level_dims(h, -1, d, None))
        self.grid = tuple(d)
        self.level_dims, self.conv_dims = [], []
        for l in range(self.nlevels + 1):
            check(lib().nsst3_level_dims(h, l, d, c))
            self.level_dims.append(tuple(d))
            self.conv_dims.append(tuple(c))
        info = (ctypes.c_int * 4)()
        self.band_info = []
        for b in range(self.nbands):
            check(lib().nsst3_band_info(h, b, info))
            self.band_info.append(tuple(info))
        self.band_level = [i[0] for i in self.band_info]
        self._grad = False
        self._fwd_token = 0   # bumped by every denoise3 call (the masks it leaves)
        # offsets of each level in the sub-band layout (64-float aligned)
        self.level_offsets = []
        off = 0
        for dims in self.level_dims:
            self.level_offsets.append(off)
            off += -(-int(np.prod(dims)) // 64) * 64
        assert off == self.subband_floats

    @property
    def handle(self):
        if self._h is None:
            raise NsstError(1, 'plan has been destroyed')
        return self._h

    def device_bytes(self):
        return lib().nsst3_plan_device_bytes(self.handle)

    def close(self):
        if self._h is not None:
            lib().nsst3_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_scalars(self, scalars):
        s = np.ascontiguousarray(scalars, dtype=np.float64).ravel()
        if s.size != self.nbands:
            raise NsstError(1, 'need %d scalars' % self.nbands)
        check(lib().nsst3_plan_set_scalars(self.handle, _dptr(s)))

    def enable_grad(self):
        """Record the threshold masks in every later denoise3 call."""
        if not self._grad:
            check(lib().nsst3_plan_enable_grad(self.handle))
            self._grad = True

    def empty_subbands(self, n=1, device=None):
        return torch.zeros((n, self.subband_floats), dtype=torch.float32, device=device or 'cuda')

    def split(self, flat):
        """(n, subband_floats) -> [level 0 (n, m0...), ..., lowpass] views."""
        out = []
        for off, dims in zip(self.level_offsets, self.level_dims):
            size = int(np.prod(dims))
            out.append(flat[:, off:off + size].unflatten(1, dims))
        return out

    def pack(self, subs):
        """Inverse of split: list of (n, *dims) tensors -> (n, subband_floats)."""
        n = subs[0].shape[0]
        flat = self.empty_subbands(n, subs[0].device)
        for off, dims, s in zip(self.level_offsets, self.level_dims, subs):
            flat[:, off:off + int(np.prod(dims))] = s.reshape(n, -1)
        return flat

    def _batch(self, x, name):
        if x.dim() == 3:
            x = x.unsqueeze(0)
        _dev(x, name)
        if tuple(x.shape[1:]) != self.shape:
            raise NsstError(1, '%s has volume shape %s, plan is for %s' % (name, tuple(x.shape[1:]), self.shape))
        if x.shape[0] > self.batch:
            raise NsstError(1, 'batch of %d exceeds the plan capacity %d' % (x.shape[0], self.batch))
        return x


def do_pyr_dec(x, plan, stream=None):
    """Band-pass pyramid: returns (flat (n, subband_floats), [bp0, ..., lowpass])."""
    x = plan._batch(x, 'x')
    flat = plan.empty_subbands(x.shape[0], x.device)
    check(lib().nsst3_pyr_dec(plan.handle, _dev(x, 'x'), _dev(flat, 'bp'), x.shape[0], _stream(stream)))
    return flat, plan.split(flat)


def do_pyr_rec(flat, plan, out=None, stream=None):
    """Pyramid reconstruction from the flat sub-band layout -> (n, n0, n1, n2)."""
    _dev(flat, 'bp')
    n = flat.shape[0]
    if out is None:
        out = torch.empty((n,) + plan.shape, dtype=torch.float32, device=flat.device)
    check(lib().nsst3_pyr_rec(plan.handle, _dev(flat, 'bp'), _dev(out, 'out'), n, _stream(stream)))
    return out


def sh_dec(flat, level, plan, stream=None):
    """Directional coefficients of one level: (n, 3*numDir^2, *level_dims)."""
    _dev(flat, 'bp')
    n = flat.shape[0]
    nb = 3 * plan.num_dirs[level] ** 2
    out = torch.empty((n, nb) + plan.level_dims[level], dtype=torch.float32, device=flat.device)
    check(lib().nsst3_sh_dec(plan.handle, _dev(flat, 'bp'), int(level), _dev(out, 'coeffs'), n, _stream(stream)))
    return out


def _thresh_args(plan, n, sigma, T, scalars):
    sig = np.ascontiguousarray(np.broadcast_to(np.asarray(sigma, np.float64), (n,)))
    t = np.ascontiguousarray(T, dtype=np.float64).ravel()
    if t.size < plan.nlevels:
        raise NsstError(1, 'T needs one multiplier per level')
    sc = None if scalars is None else np.ascontiguousarray(scalars, dtype=np.float64).ravel()
    if sc is not None and sc.size != plan.nbands:
        raise NsstError(1, 'need %d scalars' % plan.nbands)
    return sig, t, sc


def sh_dec_th_rec_cuda(flat, plan, sigma, T, scalars=None, stream=None):
    """ShDecThRec_cuda: thresholded band sums per level, lowpass copied -> flat layout."""
    _dev(flat, 'bp')
    n = flat.shape[0]
    sig, t, sc = _thresh_args(plan, n, sigma, T, scalars)
    out = torch.empty_like(flat)
    check(lib().nsst3_sh_dec_thresh_rec(plan.handle, _dev(flat, 'bp'), _dev(out, 'rec'), n, _dptr(sig), _dptr(t),
                                        None if sc is None else _dptr(sc), _stream(stream)))
    return out


def nsst_scalars3(plan, seed=0):
    """Per-band Monte-Carlo noise scalars (stored in the plan, returned as numpy)."""
    out = np.empty(plan.nbands, dtype=np.float64)
    check(lib().nsst3_compute_scalars(plan.handle, ctypes.c_uint64(seed), _dptr(out)))
    return out


def denoise3(x, plan, sigma, T=DEMO_T, scalars=None, out=None, stream=None):
    """Fused 3-D denoise of a volume or a batch of volumes (same shape out)."""
    squeeze = x.dim() == 3
    xb = plan._batch(x, 'x')
    n = xb.shape[0]
    sig, t, sc = _thresh_args(plan, n, sigma, T, scalars)
    if out is None:
        out = torch.empty_like(xb)
    ob = out.unsqueeze(0) if out.dim() == 3 else out
    check(lib().nsst3_denoise_batch(plan.handle, _dev(xb, 'x'), _dev(ob, 'out'), n, _dptr(sig), _dptr(t),
                                    None if sc is None else _dptr(sc), _stream(stream)))
    plan._fwd_token += 1
    return ob[0] if squeeze else ob


def denoise3_backward(gy, plan, out=None, stream=None):
    """d loss / d x for the volumes of the plan's most recent denoise3 call,
    given gy = d loss / d out (same shape as that call's input)."""
    squeeze = gy.dim() == 3
    gb = plan._batch(gy, 'gy')
    if out is None:
        out = torch.empty_like(gb)
    ob = out.unsqueeze(0) if out.dim() == 3 else out
    check(lib().nsst3_denoise_backward(plan.handle, _dev(gb, 'gy'), _dev(ob, 'gx'), gb.shape[0], _stream(stream)))
    return ob[0] if squeeze else ob


class Denoise3Fn(torch.autograd.Function):
    """out = denoise3(x); backward through the hand-written adjoint.  The
    plan keeps only the masks of its latest forward call, so a backward
    whose masks were overwritten first re-runs its own forward."""

    @staticmethod
    def forward(ctx, x, plan, sigma, T, scalars):
        plan.enable_grad()
        out = denoise3(x.detach().contiguous(), plan, sigma, T, scalars)
        ctx.plan, ctx.args, ctx.token = plan, (sigma, T, scalars), plan._fwd_token
        ctx.save_for_backward(x)
        return out

    @staticmethod
    def backward(ctx, gy):
        plan = ctx.plan
        (x,) = ctx.saved_tensors
        if plan._fwd_token != ctx.token:
            denoise3(x.detach().contiguous(), plan, *ctx.args)
        gx = denoise3_backward(gy.contiguous(), plan)
        return gx, None, None, None, None


def denoise3_diff(x, plan, sigma, T=DEMO_T, scalars=None):
    """Differentiable 3-D denoise (gradient with respect to the volumes)."""
    return Denoise3Fn.apply(x, plan, sigma, T, scalars)
