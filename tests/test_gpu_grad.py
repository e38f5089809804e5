"""Hand-written adjoint and gradients (differentiable denoising).

Checks, in the order of the D16 configuration's acceptance list:
  * dot-product tests <Ax, c> = <x, A^T c> and <Rc, x> = <c, R^T x>  (rel. 1e-5)
  * the GPU adjoints against the FP64 oracle adjoints               (rel-L2 1e-5)
  * grad x and grad tau against the FP64 oracle gradient             (rel-L2 1e-4)
  * grad x against FP64 central finite differences (h = 1e-3) at 32 random pixels
  * torch.autograd plumbing, batching and chunking
"""
import numpy as np
import pytest
import torch

from conftest import DCOMP, DSIZE, flat_coeffs, flat_scalars, rel_l2
from oracle import nsst2d

pytestmark = pytest.mark.gpu
_cache = {}


def _setup(H=256, W=256, batch=2):
    key = (H, W, batch)
    if key not in _cache:
        import shearcuda_gb300 as sc
        plan = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, batch=batch)
        sc.autograd.enable_grad(plan)
        sf = nsst2d.shear_spectra(H, W, DCOMP, DSIZE)
        scal = nsst2d.nsst_scalars(H, W, sf, seed=100, nthreads=8)
        _cache[key] = (plan, sf, scal)
    return _cache[key]


def _tau_lists(scal, sigma=20.0, k=3.0):
    return [k * sigma * scal[0]] + [k * sigma * np.asarray(s) for s in scal[1:]]


def _split(flat, dcomp=DCOMP):
    out, at = [flat[0]], 1
    for d in dcomp:
        out.append(flat[at:at + (1 << d)])
        at += 1 << d
    return out


def test_dot_product_tests(built_lib, cuda):
    import shearcuda_gb300 as sc
    plan, sf, scal = _setup()
    rng = np.random.default_rng(6)
    x = torch.tensor(rng.standard_normal((256, 256)), dtype=torch.float32, device=cuda)
    c = torch.tensor(rng.standard_normal((plan.nbands, 256, 256)), dtype=torch.float32, device=cuda)
    Ax = sc.shear_trans_cuda(x, 'maxflat', plan)
    Atc = sc.shear_trans_adjoint(c, plan)
    lhs = float(torch.sum(Ax.double() * c.double()))
    rhs = float(torch.sum(x.double() * Atc.double()))
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), 1.0), (lhs, rhs)
    Rc = sc.inverse_shear_cuda(c, 'maxflat', plan)
    Rtx = sc.inverse_shear_adjoint(x, plan)
    lhs = float(torch.sum(Rc.double() * x.double()))
    rhs = float(torch.sum(c.double() * Rtx.double()))
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), 1.0), (lhs, rhs)


def test_adjoints_match_oracle(built_lib, cuda):
    import shearcuda_gb300 as sc
    plan, sf, scal = _setup()
    rng = np.random.default_rng(7)
    c = rng.standard_normal((plan.nbands, 256, 256)).astype(np.float32)
    got = sc.shear_trans_adjoint(torch.tensor(c, device=cuda), plan).cpu().numpy()
    parts = [p.astype(np.float64) for p in _split(c)]
    gy = [parts[0]]
    for i in range(len(DCOMP)):
        C = np.fft.fft2(parts[i + 1], axes=(-2, -1))
        gy.append(np.real(np.fft.ifft2(np.sum(np.conj(sf[i]) * C, axis=0))))
    ref = nsst2d.atrousdec_adjoint(gy)
    assert rel_l2(got, ref) <= 1e-5
    x = rng.standard_normal((256, 256)).astype(np.float32)
    got = sc.inverse_shear_adjoint(torch.tensor(x, device=cuda), plan).cpu().numpy()
    gyp = nsst2d.atrousrec_adjoint(x.astype(np.float64), len(DCOMP))
    ref = [gyp[0]] + [np.real(np.fft.ifft2(sf[i] * np.fft.fft2(gyp[i + 1])[None], axes=(-2, -1)))
                      for i in range(len(DCOMP))]
    assert rel_l2(got, flat_coeffs(ref)) <= 1e-5


@pytest.mark.parametrize('mode', ['soft', 'hard'])
def test_gradients_match_oracle_and_finite_differences(built_lib, cuda, mode):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    plan, sf, scal = _setup()
    clean, noisy = noisy_image(256, 256, 20.0, 4)
    noisy32 = noisy.astype(np.float32)
    tau_l = _tau_lists(scal)
    tau = torch.tensor(flat_scalars(tau_l), dtype=torch.float32, device=cuda, requires_grad=True)
    x = torch.tensor(noisy32, device=cuda, requires_grad=True)
    m = 1 if mode == 'soft' else 0
    out = sc.nsst_denoise_diff(x, tau, plan, mode=m)
    loss = torch.sum((out.double() - torch.tensor(clean, device=cuda)) ** 2)
    loss.backward()
    tau64 = [np.float64(np.float32(tau_l[0]))] + [np.asarray(t, np.float32).astype(np.float64) for t in tau_l[1:]]
    l_ref, gx_ref, gt_ref = nsst2d.denoise_tau_grad(noisy32.astype(np.float64), tau64, clean, sf, mode=mode,
                                                    nthreads=8)
    assert abs(float(loss.detach()) - l_ref) <= 1e-4 * l_ref
    gx = x.grad.cpu().numpy().astype(np.float64)
    assert rel_l2(gx, gx_ref) <= 1e-4, rel_l2(gx, gx_ref)
    gt = tau.grad.cpu().numpy().astype(np.float64)
    gt_ref_flat = flat_scalars(gt_ref)
    if mode == 'soft':
        assert rel_l2(gt, gt_ref_flat) <= 1e-4, rel_l2(gt, gt_ref_flat)
    else:
        assert np.all(gt == 0.0)
    # central finite differences of the FP64 oracle at 32 random pixels.  The
    # hard rule makes the loss piecewise smooth: a pixel whose +-h step moves a
    # coefficient across its threshold sees a jump, detected by comparing
    # steps h and h/4, and is skipped (at most a few of the 32).
    rng = np.random.default_rng(5)
    x64 = noisy32.astype(np.float64)

    def fd_at(i, j, step):
        xp, xm = x64.copy(), x64.copy()
        xp[i, j] += step
        xm[i, j] -= step
        lp = np.sum((nsst2d.denoise_tau(xp, tau64, sf, mode=mode, nthreads=8)[0] - clean) ** 2)
        lm = np.sum((nsst2d.denoise_tau(xm, tau64, sf, mode=mode, nthreads=8)[0] - clean) ** 2)
        return (lp - lm) / (2 * step)

    h = 1e-3
    fd, an, skipped = [], [], 0
    for _ in range(32):
        i, j = int(rng.integers(0, 256)), int(rng.integers(0, 256))
        f1 = fd_at(i, j, h)
        if mode == 'hard':
            f2 = fd_at(i, j, h / 4)
            if abs(f1 - f2) > 1e-3 * max(1.0, abs(f2)):
                skipped += 1
                continue
        fd.append(f1)
        an.append(gx[i, j])
    fd, an = np.array(fd), np.array(an)
    assert skipped <= 4
    assert rel_l2(an, fd) <= 2e-3, (rel_l2(an, fd), np.c_[an, fd][:5])


def test_batched_and_chunked_gradients(built_lib, cuda):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    plan, sf, scal = _setup()  # capacity 2: a batch of 3 is processed in 2 chunks
    tau = torch.tensor(flat_scalars(_tau_lists(scal)), dtype=torch.float32, device=cuda)
    imgs = [noisy_image(256, 256, 20.0, 30 + i) for i in range(3)]
    x = torch.tensor(np.stack([n for _, n in imgs]).astype(np.float32), device=cuda, requires_grad=True)
    clean = torch.tensor(np.stack([c for c, _ in imgs]), device=cuda)
    t = tau.clone().requires_grad_(True)
    loss = torch.sum((sc.nsst_denoise_diff(x, t, plan).double() - clean) ** 2)
    loss.backward()
    gx_b, gt_b = x.grad.clone(), t.grad.clone()
    gt_sum = torch.zeros_like(tau)
    for i in range(3):
        xi = x.detach()[i].clone().requires_grad_(True)
        ti = tau.clone().requires_grad_(True)
        li = torch.sum((sc.nsst_denoise_diff(xi, ti, plan).double() - clean[i]) ** 2)
        li.backward()
        np.testing.assert_array_equal(xi.grad.cpu().numpy(), gx_b[i].cpu().numpy())
        gt_sum += ti.grad
    assert rel_l2(gt_b.cpu().numpy(), gt_sum.cpu().numpy()) <= 1e-5


def test_learnable_thresholds_reduce_the_loss(built_lib, cuda):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    plan, sf, scal = _setup()
    model = sc.NsstDenoiser(plan, flat_scalars(scal), 20.0, [3, 3, 3, 3, 4], device=cuda)
    imgs = [noisy_image(256, 256, 20.0, 60 + i) for i in range(2)]
    x = torch.tensor(np.stack([n for _, n in imgs]).astype(np.float32), device=cuda)
    clean = torch.tensor(np.stack([c for c, _ in imgs]).astype(np.float32), device=cuda)
    opt = torch.optim.Adam(model.parameters(), lr=0.5)
    losses = []
    for _ in range(5):
        opt.zero_grad()
        loss = torch.mean((model(x) - clean) ** 2)
        loss.backward()
        opt.step()
        losses.append(float(loss))
    assert losses[-1] < losses[0]


def test_saved_coefficients_backward_matches_recompute(built_lib, cuda):
    # the backward that reuses the forward's band spectra gives the same
    # gradients, bit for bit, as the one that recomputes them; any other
    # call on the plan drops the saved spectra
    import ctypes
    import shearcuda_gb300 as sc
    from shearcuda_gb300._lib import NsstError, THRESH_SOFT, check, lib
    from shearcuda_gb300.autograd import _ptrs
    plan, sf, scal = _setup()
    rng = np.random.default_rng(11)
    x = torch.tensor(rng.standard_normal((2, 256, 256)) * 30 + 100, dtype=torch.float32, device=cuda)
    tau = torch.tensor(flat_scalars(_tau_lists(scal)), dtype=torch.float32, device=cuda)
    xg = x.clone().requires_grad_(True)
    tg = tau.clone().requires_grad_(True)
    out = sc.nsst_denoise_diff(xg, tg, plan, THRESH_SOFT)
    assert lib().nsst_plan_saved_items(plan.handle) == 2
    gy = torch.randn_like(out)
    out.backward(gy)
    torch.cuda.synchronize()
    gx_r, gt_r = torch.empty_like(x), torch.zeros_like(tau)
    check(lib().nsst_denoise_tau_backward(plan.handle, _ptrs(x, 2), _ptrs(gy, 2), _ptrs(gx_r, 2), 2,
                                          ctypes.c_void_p(tau.data_ptr()), ctypes.c_void_p(gt_r.data_ptr()), 0,
                                          THRESH_SOFT, None))
    torch.cuda.synchronize()
    assert torch.equal(xg.grad, gx_r)
    assert torch.equal(tg.grad, gt_r)
    # the recomputing backward rewrote the arena: nothing is saved any more
    assert lib().nsst_plan_saved_items(plan.handle) == 0
    with pytest.raises(NsstError):
        check(lib().nsst_denoise_tau_backward_saved(plan.handle, _ptrs(gy, 2), _ptrs(gx_r, 2), 2,
                                                    ctypes.c_void_p(tau.data_ptr()), ctypes.c_void_p(gt_r.data_ptr()),
                                                    0, THRESH_SOFT, None))
    # a forward, then another call on the plan: the autograd backward falls back to recomputing
    xg2 = x.clone().requires_grad_(True)
    out2 = sc.nsst_denoise_diff(xg2, tau, plan, THRESH_SOFT)
    sc.shear_trans_cuda(x[0], 'maxflat', plan)
    assert lib().nsst_plan_saved_items(plan.handle) == 0
    out2.backward(gy)
    assert torch.equal(xg2.grad, gx_r)
