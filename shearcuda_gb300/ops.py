"""Python mirror of ShearCuda's GPU operator surface over libnsst.so.

Function names, argument meaning and error behaviour follow the reference's
MEX operators so that code written against them reads the same:

=============================================  =====================================================
here                                           reference (ShearCuda tree)
=============================================  =====================================================
``prepare_shearing_filters_cuda``              shearcuda/src_cuda/prepare_shearing_filters_cuda.cpp:61-249
``clear_shearing_filters_cuda``                shearcuda/src_cuda/clear_shearing_filters_cuda.cpp:51-96
``shear_trans_cuda``                           shearcuda/src_cuda/shear_trans_cuda.cpp:56-217
``thresh_cuda`` / ``softth_cuda``              shearcuda/src_cuda/thresh_cuda.cpp:57-217, softth_cuda.cpp:49-112
``inverse_shear_cuda``                         shearcuda/src_cuda/inverse_shear_cuda.cpp:57-219
``atrousdec`` / ``atrousrec``                  shearcuda/src_cuda/atrousdec.cpp:41-131, atrousrec.cpp:42-132
``nsst_scalars``                               shearlet_toolbox_1/nsst_scalars.m:28-45
``nsst_denoise``                               shearcuda/test/shear_denoise_cuda.m:14-23 (fused)
=============================================  =====================================================

Device arrays are ``torch`` CUDA float32 tensors (PyTorch supplies device
memory and streams only; all compute runs in libnsst.so's kernels).  The
coefficient "cell array" of the reference is returned as a list
``[lowpass (H, W), level 0 (ndir0, H, W), ...]`` of views into one
contiguous (nbands, H, W) tensor.  Errors raise ``NsstError`` (the
reference raises MATLAB errors through mexErrMsgTxt).
"""
import ctypes

import numpy as np
import torch

from ._lib import (NsstConfig, NsstError, NsstItem, NsstTuneResult, THRESH_HARD, THRESH_SOFT, PYRAMID_AUTO,
                   DIRECTIONAL_AUTO, DIRECTIONAL_SPLIT, DIRECTIONAL_FUSED, check, lib)

__all__ = ['ShearPlan', 'direct_support', 'prepare_shearing_filters_cuda', 'clear_shearing_filters_cuda', 'shear_trans_cuda',
           'thresh_cuda', 'softth_cuda', 'inverse_shear_cuda', 'atrousdec', 'atrousrec', 'atrousdec_noalloc',
           'nsst_scalars',
           'nsst_denoise', 'nsst_denoise_batch', 'MultiBatch', 'pyramid_filters', 'shearing_filters',
           'level_spectra', 'launch_count', 'NsstError', 'save_shearing_filters', 'load_shearing_filters', 'com_norm', 're_weight_band']


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _dev(t, name, shape=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float32:
        raise NsstError(1, '%s must be a CUDA float32 tensor' % name)
    if not t.is_contiguous():
        raise NsstError(1, '%s must be contiguous' % name)
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise NsstError(1, '%s has shape %s, expected %s' % (name, tuple(t.shape), tuple(shape)))
    return ctypes.c_void_p(t.data_ptr())


class ShearPlan:
    """The prepared shearing dictionary (the ``shear`` struct the reference's
    prepare_shearing_filters_cuda returns): filter spectra, pyramid filters
    and work buffers for one image size."""

    def __init__(self, dcomp, dsize, H, W, lpfilt='maxflat', pyramid=PYRAMID_AUTO, batch=1):
        if len(dcomp) != len(dsize):
            raise NsstError(1, 'dcomp and dsize must have the same length')
        cfg = NsstConfig()
        cfg.nlevels = len(dcomp)
        for i, (c, s) in enumerate(zip(dcomp, dsize)):
            cfg.dcomp[i] = int(c)
            cfg.dsize[i] = int(s)
        cfg.lpfilt = lpfilt.encode()
        cfg.pyramid = pyramid
        h = ctypes.c_void_p()
        check(lib().nsst_plan_create_batch(ctypes.byref(cfg), int(H), int(W), int(batch), ctypes.byref(h)))
        self._h = h
        self.dcomp, self.dsize, self.H, self.W, self.lpfilt = list(dcomp), list(dsize), int(H), int(W), lpfilt
        self.nlevels = len(dcomp)
        self.nbands = lib().nsst_plan_num_bands(h)
        lv = (ctypes.c_int * self.nbands)()
        check(lib().nsst_plan_band_levels(h, lv))
        self.band_levels = list(lv)
        self.batch = lib().nsst_plan_batch_capacity(h)

    @classmethod
    def from_file(cls, path, H, W=None, batch=1):
        """A plan over the filter bank of an SHFM0002 file (the reference's
        exported dictionary) instead of the constructed one."""
        W = H if W is None else W
        h = ctypes.c_void_p()
        check(lib().nsst_plan_create_from_file(str(path).encode(), int(H), int(W), int(batch), ctypes.byref(h)))
        self = cls.__new__(cls)
        self._h = h
        info = load_shearing_filters(path)
        self.dcomp = [int(round(np.log2(s.shape[0]))) for s in info['shear']]
        self.dsize = [s.shape[1] for s in info['shear']]
        self.H, self.W, self.lpfilt = int(H), int(W), 'file'
        self.nlevels = len(self.dcomp)
        self.nbands = lib().nsst_plan_num_bands(h)
        lv = (ctypes.c_int * self.nbands)()
        check(lib().nsst_plan_band_levels(h, lv))
        self.band_levels = list(lv)
        self.batch = lib().nsst_plan_batch_capacity(h)
        return self

    def use_graphs(self, on=True):
        check(lib().nsst_plan_use_graphs(self.handle, 1 if on else 0))

    def set_directional(self, mode):
        """'auto', 'split' or 'fused': the kernels of the directional stage of
        nsst_denoise (see nsst_plan_set_directional)."""
        m = {'auto': DIRECTIONAL_AUTO, 'split': DIRECTIONAL_SPLIT, 'fused': DIRECTIONAL_FUSED}[mode]
        check(lib().nsst_plan_set_directional(self.handle, m))

    def directional(self, n=1):
        """The directional implementation a call of n images runs: 'split' or 'fused'."""
        return {DIRECTIONAL_SPLIT: 'split', DIRECTIONAL_FUSED: 'fused'}[lib().nsst_plan_directional(self.handle, n)]

    def fused_clusters(self):
        return lib().nsst_plan_fused_clusters(self.handle)

    def autotune(self, n=1):
        """Time every directional-stage candidate on n images; the fastest
        becomes the automatic choice for batches of n's size bucket.  Returns
        {'n', 'candidates': [(name, ms)], 'chosen': name, 'direct_support',
        'direct_err', 'direct_bound_ms', 'direct_wins'} (see nsst_plan_autotune)."""
        r = NsstTuneResult()
        check(lib().nsst_plan_autotune(self.handle, int(n), ctypes.byref(r)))
        cands = [(bytes(r.name[i]).split(b'\0')[0].decode(), float(r.ms[i])) for i in range(r.ncand)]
        return {'n': r.n, 'candidates': cands, 'chosen': cands[r.chosen][0],
                'direct_support': list(r.direct_support)[:self.nlevels],
                'direct_err': list(r.direct_err)[:self.nlevels], 'direct_bound_ms': float(r.direct_bound_ms),
                'direct_wins': bool(r.direct_wins)}

    def directional_candidates(self):
        buf = ctypes.create_string_buffer(4096)
        n = lib().nsst_plan_directional_candidates(self.handle, buf, 4096)
        return buf.value.decode().split('\n')[:n]

    def select_directional(self, n, index):
        """Make candidate `index` (of directional_candidates()) the automatic
        choice for batches of n's size bucket; -1 restores the default."""
        check(lib().nsst_plan_select_directional(self.handle, int(n), int(index)))

    def check_device(self):
        """Raise NsstError(NSST_ERR_TIMEOUT) if a bounded device-side wait ran out."""
        check(lib().nsst_plan_check_device(self.handle))

    @property
    def handle(self):
        if self._h is None:
            raise NsstError(1, 'plan has been cleared')
        return self._h

    def device_bytes(self):
        return lib().nsst_plan_device_bytes(self.handle)

    def set_scalars(self, scalars):
        s = np.ascontiguousarray(flatten_scalars(scalars), dtype=np.float64)
        if s.size != self.nbands:
            raise NsstError(1, 'need %d scalars' % self.nbands)
        check(lib().nsst_plan_set_scalars(self.handle, _dptr(s)))

    def level_spectra(self, level):
        nd = 1 << self.dcomp[level]
        out = np.empty((nd, self.H, self.W // 2 + 1), dtype=np.complex128)
        check(lib().nsst_plan_level_spectra(self.handle, level, _dptr(out.view(np.float64))))
        return out

    def enable_timers(self, on=True):
        check(lib().nsst_timers_enable(self.handle, 1 if on else 0))

    def read_timers(self, max_stages=32):
        """Per-stage milliseconds of the last execute call, as [(name, ms)]."""
        names = ctypes.create_string_buffer(4096)
        ms = (ctypes.c_float * max_stages)()
        n = lib().nsst_timers_read(self.handle, names, 4096, ms, max_stages)
        if n < 0:
            raise NsstError(4, 'timer read failed')
        labels = names.value.decode().split('\n')[:n]
        return list(zip(labels, [float(ms[i]) for i in range(n)]))

    def close(self):
        if self._h is not None:
            lib().nsst_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def split(self, coeffs):
        """(nbands, H, W) tensor -> [lowpass, level0 (ndir0,H,W), ...] views."""
        out = [coeffs[0]]
        at = 1
        for c in self.dcomp:
            out.append(coeffs[at:at + (1 << c)])
            at += 1 << c
        return out


def flatten_scalars(scalars):
    """Accept the reference's cell layout {lowpass, [per-direction]...} or a flat list."""
    if isinstance(scalars, (list, tuple)) and len(scalars) and np.ndim(scalars[0]) == 0 and \
            any(np.ndim(s) > 0 for s in scalars[1:]):
        return np.concatenate([np.atleast_1d(np.asarray(s, np.float64)) for s in scalars])
    return np.asarray(scalars, dtype=np.float64).ravel()


def _kvec(plan, K):
    K = np.ascontiguousarray(np.asarray(K, dtype=np.float64).ravel())
    if K.size == 3 and plan.nlevels != 2:
        # nsst_HT.m Tscalars: [lowpass, levels 1..J-1, finest level J]
        K = np.array([K[0]] + [K[1]] * (plan.nlevels - 1) + [K[2]], dtype=np.float64)
    if K.size != plan.nlevels + 1:
        raise NsstError(1, 'K needs nlevels+1 (or 3, Tscalars-style) entries')
    return K


def prepare_shearing_filters_cuda(dcomp, dsize, H, W=None, lpfilt='maxflat', pyramid=PYRAMID_AUTO, batch=1):
    return ShearPlan(dcomp, dsize, H, H if W is None else W, lpfilt, pyramid, batch)


def clear_shearing_filters_cuda(shear):
    shear.close()


def atrousdec(x, shear, stream=None):
    y = torch.empty((shear.nlevels + 1, shear.H, shear.W), device=x.device, dtype=torch.float32)
    check(lib().nsst_atrousdec(shear.handle, _dev(x, 'x', (shear.H, shear.W)), _dev(y, 'y'), _stream(stream)))
    return y


def atrousrec(y, shear, stream=None):
    x = torch.empty((shear.H, shear.W), device=y.device, dtype=torch.float32)
    check(lib().nsst_atrousrec(shear.handle, _dev(y, 'y', (shear.nlevels + 1, shear.H, shear.W)), _dev(x, 'x'),
                               _stream(stream)))
    return x


def atrousdec_noalloc(x, nlevels, y, lpfilt='maxflat', stream=None):
    """À trous analysis through the entry point that allocates no device
    memory (for callers that cannot call cudaMalloc): ``y`` must be a
    preallocated (nlevels+1, H, W) CUDA float32 tensor; at most 2048*2048
    pixels; calls overlapping on the GPU race on the library's one scratch image."""
    H, W = x.shape
    check(lib().nsst_atrousdec_noalloc(_dev(x, 'x'), _dev(y, 'y', (nlevels + 1, H, W)), H, W, nlevels,
                                       lpfilt.encode(), _stream(stream)))
    return y


def _check_lpfilt(lpfilt, shear):
    # a dictionary read from a filter-bank file carries its own pyramid filters
    if shear.lpfilt != 'file' and lpfilt != shear.lpfilt:
        raise NsstError(1, 'lpfilt %r does not match the prepared dictionary (%r)' % (lpfilt, shear.lpfilt))


def shear_trans_cuda(x, lpfilt, shear, coeff=None, stream=None):
    """Forward NSST.  ``coeff`` (optional) is written in place, like the
    reference's coeff_inplace argument (shear_trans_cuda.cpp:191-205)."""
    _check_lpfilt(lpfilt, shear)
    if coeff is None:
        coeff = torch.empty((shear.nbands, shear.H, shear.W), device=x.device, dtype=torch.float32)
    check(lib().nsst_shear_trans(shear.handle, _dev(x, 'x', (shear.H, shear.W)),
                                 _dev(coeff, 'coeff', (shear.nbands, shear.H, shear.W)), _stream(stream)))
    return coeff


def thresh_cuda(coeff, sigma, K, scalars, shear, mode=THRESH_HARD, stream=None, opt=0):
    """In-place threshold of all bands: t_b = K[level(b)] * sigma * scalars[b].
    opt == 1 returns, like the reference's thresh_cuda, the largest thresholded
    magnitude relative to its band scalar (max_b max|c_b| / scalars[b]);
    otherwise the coefficients."""
    s = np.ascontiguousarray(flatten_scalars(scalars), dtype=np.float64)
    if s.size != shear.nbands:
        raise NsstError(1, 'need %d scalars' % shear.nbands)
    K = _kvec(shear, K)
    c = _dev(coeff, 'coeff', (shear.nbands, shear.H, shear.W))
    if opt == 1:
        m = ctypes.c_double()
        check(lib().nsst_thresh_max(shear.handle, c, float(sigma), _dptr(K), _dptr(s), mode, ctypes.byref(m),
                                    _stream(stream)))
        return m.value
    check(lib().nsst_thresh(shear.handle, c, float(sigma), _dptr(K), _dptr(s), mode, _stream(stream)))
    return coeff


def re_weight_band(P, coeff, shear, out=None, stream=None):
    """Image re-synthesised with a weight per pyramid band (re_weight_band.m):
    len(coeff) - 1 pyramid levels (at most the plan's), coeff[0] on the
    lowpass, coeff[1:] on the band-pass images coarse to fine."""
    w = np.ascontiguousarray(coeff, dtype=np.float64).ravel()
    x = _dev(P, 'P', (shear.H, shear.W))
    if out is None:
        out = torch.empty_like(P)
    check(lib().nsst_re_weight_band(shear.handle, x, _dptr(w), int(w.size), _dev(out, 'out', (shear.H, shear.W)),
                                    _stream(stream)))
    return out


def com_norm(shear):
    """Exact l2 norms of the shearlets of every band (com_norm.m:25-55), in
    coefficient plane order; usable as thresh_cuda's scalars."""
    out = np.empty(shear.nbands, dtype=np.float64)
    check(lib().nsst_band_norms(shear.handle, _dptr(out)))
    return out


def softth_cuda(coeff, sigma, K, scalars, shear, stream=None):
    return thresh_cuda(coeff, sigma, K, scalars, shear, THRESH_SOFT, stream)


def inverse_shear_cuda(coeff, lpfilt, shear, stream=None):
    _check_lpfilt(lpfilt, shear)
    x = torch.empty((shear.H, shear.W), device=coeff.device, dtype=torch.float32)
    check(lib().nsst_inverse_shear(shear.handle, _dev(coeff, 'coeff', (shear.nbands, shear.H, shear.W)),
                                   _dev(x, 'x'), _stream(stream)))
    return x


def nsst_denoise(x, shear, sigma, K, scalars=None, mode=THRESH_HARD, out=None, stream=None):
    if out is None:
        out = torch.empty_like(x)
    K = _kvec(shear, K)
    sp = None
    if scalars is not None:
        s = np.ascontiguousarray(flatten_scalars(scalars), dtype=np.float64)
        if s.size != shear.nbands:
            raise NsstError(1, 'need %d scalars' % shear.nbands)
        sp = _dptr(s)
    check(lib().nsst_denoise(shear.handle, _dev(x, 'x', (shear.H, shear.W)), _dev(out, 'out', (shear.H, shear.W)),
                             float(sigma), _dptr(K), sp, mode, _stream(stream)))
    return out


def _ptr_array(ts, name, shape):
    arr = (ctypes.c_void_p * len(ts))()
    for i, t in enumerate(ts):
        arr[i] = _dev(t, '%s[%d]' % (name, i), shape).value
    return arr


def nsst_denoise_batch(xs, shear, sigmas, K, scalars=None, mode=THRESH_HARD, outs=None, stream=None):
    """Denoise a list of same-size images in one batched pass."""
    n = len(xs)
    if outs is None:
        outs = [torch.empty_like(x) for x in xs]
    K = _kvec(shear, K)
    sg = np.ascontiguousarray(np.broadcast_to(np.asarray(sigmas, np.float64), (n,)))
    sp = None
    if scalars is not None:
        s = np.ascontiguousarray(flatten_scalars(scalars), dtype=np.float64)
        if s.size != shear.nbands:
            raise NsstError(1, 'need %d scalars' % shear.nbands)
        sp = _dptr(s)
    check(lib().nsst_denoise_batch(shear.handle, _ptr_array(xs, 'x', (shear.H, shear.W)),
                                   _ptr_array(outs, 'out', (shear.H, shear.W)), n, _dptr(sg), _dptr(K), sp, mode,
                                   _stream(stream)))
    return outs


class MultiBatch:
    """Uneven batch over several plans (one per image size), replayed as one CUDA graph."""

    def __init__(self, plans):
        self.plans = list(plans)
        arr = (ctypes.c_void_p * len(self.plans))(*[p.handle.value for p in self.plans])
        h = ctypes.c_void_p()
        check(lib().nsst_multi_create(arr, len(self.plans), ctypes.byref(h)))
        self._h = h
        self._index = {(p.H, p.W): i for i, p in enumerate(self.plans)}

    def denoise(self, xs, sigmas, K, mode=THRESH_HARD, outs=None, stream=None):
        n = len(xs)
        if outs is None:
            outs = [torch.empty_like(x) for x in xs]
        items = (NsstItem * n)()
        for i, (x, o, s) in enumerate(zip(xs, outs, sigmas)):
            pi = self._index.get(tuple(x.shape))
            if pi is None:
                raise NsstError(1, 'no plan for image size %s' % (tuple(x.shape),))
            items[i].x = _dev(x, 'x').value
            items[i].out = _dev(o, 'out', tuple(x.shape)).value
            items[i].sigma = float(s)
            items[i].plan = pi
        K = _kvec(self.plans[0], K)
        check(lib().nsst_multi_denoise(self._h, items, n, _dptr(K), mode, _stream(stream)))
        return outs

    def close(self):
        if self._h is not None:
            lib().nsst_multi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def direct_support(dcomp, dsize, H, W, tol=1e-5):
    """Per level: the smallest square window (px) of the effective spatial
    directional filters keeping the truncation error <= tol (0: none below the
    image size), and the worst band's error there (host only, no GPU)."""
    cfg = NsstConfig()
    cfg.nlevels = len(dcomp)
    for i, (c, s) in enumerate(zip(dcomp, dsize)):
        cfg.dcomp[i] = int(c)
        cfg.dsize[i] = int(s)
    cfg.lpfilt = b'maxflat'
    sup = (ctypes.c_int * len(dcomp))()
    err = (ctypes.c_double * len(dcomp))()
    check(lib().nsst_direct_support(ctypes.byref(cfg), int(H), int(W), float(tol), sup, err))
    return list(sup), list(err)


def launch_count():
    """Kernels launched by libnsst.so since it was loaded."""
    return int(lib().nsst_launch_count())


def nsst_scalars(shear, seed=0):
    out = np.empty(shear.nbands, dtype=np.float64)
    check(lib().nsst_compute_scalars(shear.handle, ctypes.c_uint64(seed), _dptr(out)))
    return out


# ------------------------------------------------------------ host-only helpers
def save_shearing_filters(m, num, data_type='single', path=None, lpfilt='maxflat'):
    """Write the filter bank of dsize m / dcomp num as the reference's
    SHFM0002 file (save_shearing_filters.m:46-84); the default file name is
    the reference's, shearFilters_<num..>_<data_type>.bin.  Returns the path."""
    if len(m) != len(num):
        raise NsstError(1, 'm and num must have the same length')
    if data_type not in ('single', 'double'):
        raise NsstError(1, "data_type must be 'single' or 'double'")
    if path is None:
        path = 'shearFilters' + ''.join('_%d' % v for v in num) + '_' + data_type + '.bin'
    cfg = NsstConfig()
    cfg.nlevels = len(num)
    for i, (c, sz) in enumerate(zip(num, m)):
        cfg.dcomp[i] = int(c)
        cfg.dsize[i] = int(sz)
    cfg.lpfilt = lpfilt.encode()
    check(lib().nsst_filters_save(str(path).encode(), ctypes.byref(cfg), 0 if data_type == 'single' else 2))
    return path


def load_shearing_filters(path):
    """Read an SHFM0002 file: {'data_type', 'shear': [(ndir, n, n) per scale],
    'atrous': [h0, h1, g0, g1]} as FP64 arrays (row-major)."""
    nl = ctypes.c_int()
    ds, nd = (ctypes.c_int * 8)(), (ctypes.c_int * 8)()
    F, dt = (ctypes.c_int * 4)(), ctypes.c_int()
    check(lib().nsst_filters_load(str(path).encode(), ctypes.byref(nl), ds, nd, F, None, None, ctypes.byref(dt)))
    shear = np.empty(sum(nd[l] * ds[l] ** 2 for l in range(nl.value)), np.float64)
    pyr = np.empty(sum(f * f for f in F), np.float64)
    check(lib().nsst_filters_load(str(path).encode(), ctypes.byref(nl), ds, nd, F, _dptr(shear), _dptr(pyr), None))
    out, at = [], 0
    for l in range(nl.value):
        k = nd[l] * ds[l] ** 2
        out.append(shear[at:at + k].reshape(nd[l], ds[l], ds[l]))
        at += k
    atr, at = [], 0
    for f in F:
        atr.append(pyr[at:at + f * f].reshape(f, f))
        at += f * f
    return {'data_type': 'single' if dt.value == 0 else 'double', 'shear': out, 'atrous': atr}


def pyramid_filters(name='maxflat'):
    F = (ctypes.c_int * 4)()
    check(lib().nsst_pyramid_filters(name.encode(), F, None))
    taps = np.empty(sum(f * f for f in F), dtype=np.float64)
    check(lib().nsst_pyramid_filters(name.encode(), F, _dptr(taps)))
    out, at = [], 0
    for f in F:
        out.append(taps[at:at + f * f].reshape(f, f))
        at += f * f
    return tuple(out)


def shearing_filters(n1, level):
    out = np.empty((1 << level, n1, n1), dtype=np.float64)
    check(lib().nsst_shearing_filters(n1, level, _dptr(out)))
    return out


def level_spectra(dsize, dcomp, H, W):
    out = np.empty((1 << dcomp, H, W // 2 + 1), dtype=np.complex128)
    check(lib().nsst_level_spectra(dsize, dcomp, H, W, _dptr(out.view(np.float64))))
    return out
