"""Benchmark: NSST decompose + hard threshold + reconstruct, images/s.

Default workload (N=1): a batch of 64 synthetic 512x512 images denoised in
one batched pass per step (dcomp [3 3 4 4], dsize [32 32 16 16], maxflat
pyramid, K = [0 3 3 3 4], sigma 20).  `value` times the batched pass with
inputs already in HBM (CUDA events on the launching stream, L2 flushed
between steps); `e2e` times the same pass through the public C ABI with the
host->device copy of the inputs and the device->host copy of the outputs in
the timed region.  Extra keys report the plain one-image-per-call path, the
uneven 64-image batch (sizes from {256^2, 384x512, 512^2, 768x1024, 1024^2})
and the per-stage roofline of the dominant kernel.

`--impl reference` times the reference's CPU path (the FP64 oracle port of
nsst_dec2 / nsst_HT / nsst_rec2 with the C restatement of atrousc.cpp) on the
host cores instead.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DCOMP, DSIZE, K = [3, 3, 4, 4], [32, 32, 16, 16], [0, 3, 3, 3, 4]
H = W = 512
BATCH = 64
SIGMA = 20.0
METRIC = 'NSST dec+thresh+rec images/s at 512^2 fp32, batched'
UNIT = 'images/s'


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=50)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--no-extras', action='store_true', help='skip the plain/uneven/e2e extras')
    ap.add_argument('--batch', type=int, default=BATCH, help='images per batched pass (smaller for profiling)')
    ap.add_argument('--size', default='%dx%d' % (H, W),
                    help='HxW of the batched pass\'s images in the 2-D workload of the gb300 arm (other sizes '
                         'for profiling their kernels; use with --no-extras)')
    ap.add_argument('--workload', default='2d', choices=['2d', 'v3', 'sep'],
                    help="v3 / sep: only the 3-D volume or the image-separation extra (for profiling their kernels)")
    ap.add_argument('--sep-batch', type=int, default=8, help='images per batched separation call')
    ap.add_argument('--v3-sizes', default='128,192', help='volume edge lengths of the v3 workload')
    ap.add_argument('--v3-batch', type=int, default=4, help='volumes per batched v3 pass')
    ap.add_argument('--directional', default='auto',
                    help='directional-stage kernels of the batched pass: the autotuner\'s choice (auto, the plan is '
                         'tuned for the batch first), split or fused (the plan\'s untuned choice of that kind), or '
                         'one autotuner candidate by name, e.g. split/level/rows8/synthesis (for profiling it)')
    ap.add_argument('--cpu-sweep', action='store_true',
                    help='only the CPU baseline table: the FP64 oracle port at 512^2, 1024^2 and 2048^2, one thread '
                         'and all host threads (median of 5 / 5 / 3 runs); no GPU work')
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


def max_over_ranks(value, device):
    """The largest of every rank's value (the slowest replica times the job);
    the value itself on a single process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, seconds):
    """Whole-job units/s: every replica processes units_per_rank in the job time."""
    return units_per_rank * world / seconds


# --------------------------------------------------------------- CPU baseline
def cpu_baseline(min_seconds=10.0, max_images=8):
    """The oracle (FP64 NumPy/SciPy + C atrous restatement) on the host cores,
    on a bounded sample of the same workload: whole images of the batch's
    size, one at a time, until min_seconds have passed; and one image on a
    single thread."""
    from oracle import nsst2d
    from shearcuda_gb300.synth import noisy_image
    cores = os.cpu_count() or 1
    sf = nsst2d.shear_spectra(H, W, DCOMP, DSIZE)
    scal = nsst2d.nsst_scalars(H, W, sf, seed=100, nthreads=cores)
    n = 0
    t0 = time.perf_counter()
    while n < max_images:
        _, noisy = noisy_image(H, W, SIGMA, n)
        nsst2d.denoise(noisy, SIGMA, K, scal, DCOMP, DSIZE, shear_f=sf, nthreads=cores)
        n += 1
        if time.perf_counter() - t0 >= min_seconds:
            break
    dt = time.perf_counter() - t0
    _, noisy = noisy_image(H, W, SIGMA, 0)
    t1 = time.perf_counter()
    nsst2d.denoise(noisy, SIGMA, K, scal, DCOMP, DSIZE, shear_f=sf, nthreads=1)
    one = time.perf_counter() - t1
    return {'value': n / dt, 'unit': UNIT, 'cores': cores, 'kind': 'port',
            'sample': '%d of the %dx%d images, dec+thresh+rec, filter/scalar setup excluded, %.1f s' % (n, H, W, dt),
            'single_thread': {'value': 1.0 / one, 'unit': UNIT, 'cores': 1,
                              'sample': 'one %dx%d image, %.1f s' % (H, W, one)}}


def cpu_sweep():
    """The CPU baseline table: the oracle port's dec + hard threshold + rec
    per image at 512^2, 1024^2 and 2048^2 (seeds 0, 1, 2, sigma 20), on one
    thread and on every host thread (median of 5, 5 and 3 runs), filter and
    scalar setup timed separately."""
    from oracle import nsst2d
    from shearcuda_gb300.synth import noisy_image
    cores = os.cpu_count() or 1
    rows = []
    for (H_, W_), seed, reps in (((512, 512), 0, 5), ((1024, 1024), 1, 5), ((2048, 2048), 2, 3)):
        t0 = time.perf_counter()
        sf = nsst2d.shear_spectra(H_, W_, DCOMP, DSIZE)
        scal = nsst2d.nsst_scalars(H_, W_, sf, seed=100, nthreads=cores)
        setup = time.perf_counter() - t0
        _, noisy = noisy_image(H_, W_, SIGMA, seed)
        row = {'H': H_, 'W': W_, 'setup_s': setup}
        for nt in (1, cores):
            ts = []
            for _ in range(reps):
                t1 = time.perf_counter()
                nsst2d.denoise(noisy, SIGMA, K, scal, DCOMP, DSIZE, shear_f=sf, nthreads=nt)
                ts.append(time.perf_counter() - t1)
            row['threads_%d' % nt] = {'median_s': float(np.median(ts)), 'runs': reps,
                                      'images_per_s': 1.0 / float(np.median(ts))}
        rows.append(row)
        print(json.dumps({'cpu_sweep_row': row}), flush=True)
    print(json.dumps({'workload': 'cpu_sweep', 'cores': cores, 'kind': 'port', 'rows': rows}), flush=True)


def run_reference(args):
    """Each step denoises one 512x512 image of the batch on the host cores
    (a bounded sample of the 64-image workload); rank 0 only."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import nsst2d
    from shearcuda_gb300.synth import noisy_image
    cores = os.cpu_count() or 1
    sf = nsst2d.shear_spectra(H, W, DCOMP, DSIZE)
    scal = nsst2d.nsst_scalars(H, W, sf, seed=100, nthreads=cores)
    steps = max(1, min(args.steps, 60))
    for i in range(min(args.warmup, 1)):
        _, noisy = noisy_image(H, W, SIGMA, 10000 + i)
        nsst2d.denoise(noisy, SIGMA, K, scal, DCOMP, DSIZE, shear_f=sf, nthreads=cores)
    t0 = time.perf_counter()
    for i in range(steps):
        _, noisy = noisy_image(H, W, SIGMA, i)
        nsst2d.denoise(noisy, SIGMA, K, scal, DCOMP, DSIZE, shear_f=sf, nthreads=cores)
    dt = time.perf_counter() - t0
    v = steps / dt
    cb = {'value': v, 'unit': UNIT, 'cores': cores, 'kind': 'port',
          'sample': '%d of the 512x512 images (one per step), dec+thresh+rec in FP64, setup excluded' % steps}
    line = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': UNIT, 'n_gpus': world,
            'steps': steps, 'warmup': args.warmup, 'ms_per_step': 1000.0 * dt / steps,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': 'reference CPU path (FP64 oracle port of nsst_dec2/nsst_HT/nsst_rec2 + atrousc '
                                   'restatement), one 512x512 image of the 64-image batch per step',
                       'H': H, 'W': W, 'dcomp': DCOMP, 'dsize': DSIZE, 'K': K},
            'cpu_baseline': cb,
            'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- clock sampler
class ClockSampler:
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.FIELDS,
                                          '--format=csv,noheader,nounits', '-lms', '50'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(',')])

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for r in self.rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower() == 'active':
                    reasons.add(nm)
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


# --------------------------------------------------------------- GPU arm
def measured_peak():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback'


# Stage groups of the library's per-stage timers, mapped to the terms of the
# fused design's algorithmic traffic (per image of N pixels, FP32): pyramid
# analysis 48N B (4 levels x read 1 + write 2 images), directional 32N B
# (4 levels x read the band-pass level + write its band sum) plus the filter
# spectra, 192N B, once per distinct size per launch, synthesis 48N B.
STAGE_GROUPS = {
    'pyramid_analysis': ('dct_rows_image', 'dct_cols_image', 'dct_rows_levels', 'dct_cols_levels',
                         'dct_lowpass_threshold', 'fft_rows_fwd', 'fft_cols_fwd'),
    'directional': ('band_analysis_cols', 'band_rows_threshold', 'band_synthesis_cols', 'band_fused'),
    'synthesis': ('dct_cols_sums', 'dct_rows_synthesis', 'dct_cols_image_out', 'fft_rows_inv', 'lowpass_threshold'),
}


def s8d_bytes(nimg, H_, W_):
    """Algorithmic HBM bytes of one pass over nimg images of one size, per
    stage group (the spectra counted once per launch)."""
    N = H_ * W_
    return {'pyramid_analysis': 48 * N * nimg, 'directional': 32 * N * nimg + 192 * N, 'synthesis': 48 * N * nimg}


def fft_flops(nimg, H_, W_, ntrans=104):
    """FP32 flops of the pass's 2-D real FFTs: per image 4 level transforms,
    48 band inverses, 48 band forwards and 4 level inverses, 2.5 N log2 N each."""
    N = H_ * W_
    return nimg * ntrans * 2.5 * N * np.log2(N)


def fp32_peak_tflops(sm_count):
    """Nominal FP32 FMA peak: SMs x 128 lanes x 2 flop x the maximum SM clock
    (MEASURED_PEAKS.json's sm_max_mhz, else 2070 MHz)."""
    mhz = 2070.0
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            mhz = float(json.load(f).get('sm_max_mhz', mhz))
    except (OSError, ValueError):
        pass
    return sm_count * 128 * 2 * mhz * 1e6 / 1e12


def roofline_report(stage_ms, nimg, H_, W_, peak, peak_kind, ms_per_step, sm_count, traffic_db=None):
    """The roofline object of the bench line: the directional stage (the
    dominant one) against the HBM peak with the fused design's algorithmic
    bytes, the same for the whole step and each stage group, and the FFT
    arithmetic against the FP32 peak."""
    alg = s8d_bytes(nimg, H_, W_)
    groups = {}
    for g, names in STAGE_GROUPS.items():
        ms = sum(stage_ms.get(k, 0.0) for k in names)
        if ms > 0:
            a = alg[g] / (ms / 1000.0) / 1e9
            groups[g] = {'ms': ms, 'algorithmic_bytes': alg[g], 'achieved_gbs': a, 'frac': a / peak}
    d = groups.get('directional', {'ms': float('nan'), 'achieved_gbs': float('nan')})
    step_bytes = sum(alg.values())
    step_gbs = step_bytes / (ms_per_step / 1000.0) / 1e9
    traffic, ratio = None, None
    if traffic_db:
        parts = [traffic_db[k] for k in STAGE_GROUPS['directional'] if k in stage_ms and k in traffic_db]
        if parts and len(parts) == sum(1 for k in STAGE_GROUPS['directional'] if k in stage_ms):
            traffic = float(sum(parts)) * nimg / traffic_db.get('_images', nimg)
            ratio = traffic / alg['directional']
    fl = fft_flops(nimg, H_, W_)
    pk = fp32_peak_tflops(sm_count)
    ach = fl / (ms_per_step / 1000.0) / 1e12
    return {'bound': 'hbm', 'achieved': d['achieved_gbs'], 'peak': peak, 'unit': 'GB/s',
            'frac': d['achieved_gbs'] / peak, 'traffic': traffic, 'traffic_ratio': ratio,
            'kernel': 'directional stage (%s)' % ' + '.join(k for k in STAGE_GROUPS['directional'] if k in stage_ms),
            'kernel_ms': d['ms'], 'algorithmic_bytes_per_launch': alg['directional'], 'peak_source': peak_kind,
            'step': {'algorithmic_bytes': step_bytes, 'achieved_gbs': step_gbs, 'frac': step_gbs / peak},
            'stage_groups': groups,
            'compute': {'bound': 'fp32', 'fft_flops_per_step': fl, 'achieved_tflops': ach, 'peak_tflops': pk,
                        'frac': ach / pk, 'peak_source': 'nominal (SMs x 128 FP32 lanes x 2 x max SM clock)'},
            'stages_ms': stage_ms}


def algorithmic_bytes(stage, nimg, H_, W_, nlev=4, nbands_dir=48):
    """Bytes one launch of a split-pipeline stage moves as designed (band
    planes materialised: FP32 real images 4 B/px, packed spectra 8 B per 2 px);
    reported beside the fused design's algorithmic bytes (s8d_bytes)."""
    N = H_ * W_
    per = {
        # band round trip: read the band's packed spectrum and write it back
        'band_rows_threshold': 8 * N * nbands_dir,
        # read the level spectrum once per band (L2-shared) + write the band
        'band_analysis_cols': 4 * N * nbands_dir + 4 * N * nlev,
        # read every band once, write the level sum
        'band_synthesis_cols': 4 * N * nbands_dir + 4 * N * nlev,
        'fft_rows_fwd': 8 * N * nlev, 'fft_cols_fwd': 8 * N * nlev, 'fft_rows_inv': 8 * N * nlev,
        # the spectral pyramid (FP32 planes, 4 B/px; packed spectra 4 B/px)
        'dct_rows_image': 8 * N, 'dct_cols_image': 8 * N, 'dct_cols_image_out': 8 * N,
        'dct_rows_levels': 8 * N * nlev, 'dct_cols_levels': 8 * N * nlev, 'dct_cols_sums': 8 * N * nlev,
        'dct_rows_synthesis': (4 * nlev + 8) * N,
    }
    if stage.startswith('atrous_dec'):
        return 8 * N * nimg  # read the lowpass, write one output
    if stage.startswith('atrous_rec'):
        return 12 * N * nimg  # read two inputs, write one output
    b = per.get(stage, 0) * nimg
    # spectra: read once per launch (shared by the batch) where used
    if stage in ('band_analysis_cols', 'band_synthesis_cols'):
        b += 4 * N * nbands_dir
    # level response tables: read once per launch
    if stage == 'dct_rows_levels':
        b += 4 * N * nlev
    if stage == 'dct_rows_synthesis':
        b += 4 * N * (nlev + 1)
    return b


def volume_bench(sc, torch, dev, stream, flush, rank, reps=3, sizes=(128, 192), batch=4):
    """3-D denoise of seeded ellipsoid sequences (sigma 30, T = [3.3 3 3]):
    volumes/s of the batched forward and of forward + adjoint (gradient with
    respect to the volumes at the forward's threshold masks)."""
    from shearcuda_gb300.synth import noisy_volume
    out = {'num_dirs': list(sc.V3_NUM_DIRS), 'T': list(sc.DEMO_T[:3]), 'sigma': 30.0}
    for n in sizes:
        p = sc.VolumePlan(n, n, n, num_dirs=sc.V3_NUM_DIRS, batch=batch)
        sc.nsst_scalars3(p, seed=9)
        p.enable_grad()
        xb = torch.stack([torch.tensor(noisy_volume((n, n, n), 30.0, 500 * rank + i)[1].astype(np.float32),
                                       device=dev) for i in range(batch)])
        ob = torch.empty_like(xb)
        gy = torch.randn_like(xb)
        gx = torch.empty_like(xb)

        def fwd():
            sc.denoise3(xb, p, 30.0, sc.DEMO_T, out=ob)

        def fwd_bwd():
            fwd()
            sc.denoise3_backward(gy, p, out=gx)

        res = {'grid': p.grid[0], 'conv_lengths': [c[0] for c in p.conv_dims[:3]],
               'device_bytes': p.device_bytes()}
        c0 = sc.launch_count()
        fwd()
        res['kernels_forward'] = sc.launch_count() - c0
        for name, f in (('forward_ms', fwd), ('forward_adjoint_ms', fwd_bwd)):
            for _ in range(2):
                f()
            torch.cuda.synchronize()
            tt = 0.0
            for _ in range(reps):
                flush.fill_(1.0)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                f()
                e1.record(stream)
                torch.cuda.synchronize()
                tt += e0.elapsed_time(e1)
            res[name] = tt / reps
        res['volumes_per_s'] = batch / (res['forward_ms'] / 1000.0)
        res['ratio'] = res['forward_adjoint_ms'] / res['forward_ms']
        p.close()
        # the same forward on the reference's padding (MarshalData.m: 128 -> 132, 192 -> 204)
        pm = sc.VolumePlan(n, n, n, num_dirs=sc.V3_NUM_DIRS, batch=batch, grid='marshal')
        sc.nsst_scalars3(pm, seed=9)
        for _ in range(2):
            sc.denoise3(xb, pm, 30.0, sc.DEMO_T, out=ob)
        torch.cuda.synchronize()
        tt = 0.0
        for _ in range(reps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sc.denoise3(xb, pm, 30.0, sc.DEMO_T, out=ob)
            e1.record(stream)
            torch.cuda.synchronize()
            tt += e0.elapsed_time(e1)
        res['marshal_grid'] = {'grid': pm.grid[0], 'forward_ms': tt / reps,
                               'volumes_per_s': batch / (tt / reps / 1000.0)}
        pm.close()
        out['b%dx%d' % (batch, n)] = res
        del xb, ob, gy, gx
    return out


SEP_DCOMP, SEP_DSIZE, SEP_N = [3, 3, 4, 4], [80, 80, 80, 80], 256
SEP_ARGS = dict(level2=4, itermax=10, stop=3.0, gamma=3.0, coeff=[.1, .1, 1.5, 1.5])


def separation_bench(sc, torch, dev, stream, flush, rank, reps=5, batch=8, cpu_sample=True):
    """The separation demo's configuration (separation_demo01_gpu.m:19-41, 80):
    256x256 points + curves images (150 points, sigma 20), shearlets dcomp
    [3 3 4 4] dsize [80 80 80 80], level2 4, itermax 10, stop 3, gamma 3,
    coeff [.1 .1 1.5 1.5]; one batched nsst_separate call per step (setup with
    its host reductions + the 10 iterations)."""
    from shearcuda_gb300.synth import points_and_curves
    host = [points_and_curves(SEP_N, npoints=150, sigma=20.0, seed=700 * rank + i)[1].astype(np.float32)
            for i in range(batch)]
    plan = sc.prepare_shearing_filters_cuda(SEP_DCOMP, SEP_DSIZE, SEP_N, SEP_N, batch=batch)
    x = torch.tensor(np.stack(host), device=dev)
    out = {'batch': batch, 'H': SEP_N, 'W': SEP_N, 'dcomp': SEP_DCOMP, 'dsize': SEP_DSIZE, **SEP_ARGS}
    c0 = sc.launch_count()
    sc.separate(x, shear=plan, **SEP_ARGS)
    torch.cuda.synchronize()
    out['kernels_per_call'] = sc.launch_count() - c0
    for _ in range(2):
        sc.separate(x, shear=plan, **SEP_ARGS)
    torch.cuda.synchronize()
    tt = 0.0
    for _ in range(reps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sc.separate(x, shear=plan, **SEP_ARGS)
        e1.record(stream)
        torch.cuda.synchronize()
        tt += e0.elapsed_time(e1)
    out['ms_per_call'] = tt / reps
    out['images_per_s'] = batch / (out['ms_per_call'] / 1000.0)
    # split: one iteration's cost from itermax 10 vs 1, the rest is the setup
    one = dict(SEP_ARGS, itermax=1)
    sc.separate(x, shear=plan, **one)
    t1 = 0.0
    for _ in range(reps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sc.separate(x, shear=plan, **one)
        e1.record(stream)
        torch.cuda.synchronize()
        t1 += e0.elapsed_time(e1)
    t1 /= reps
    out['ms_per_iteration'] = (out['ms_per_call'] - t1) / (SEP_ARGS['itermax'] - 1)
    out['ms_setup'] = t1 - out['ms_per_iteration']
    # e2e: pinned host images in, both parts out, inside the timed region
    pin_in = torch.from_numpy(np.stack(host)).pin_memory()
    pin_c = torch.empty_like(pin_in).pin_memory()
    pin_p = torch.empty_like(pin_in).pin_memory()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        x.copy_(pin_in, non_blocking=True)
        C, P, _ = sc.separate(x, shear=plan, **SEP_ARGS)
        pin_c.copy_(C, non_blocking=True)
        pin_p.copy_(P, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / reps
    out['e2e'] = {'value': batch / (e2e_ms / 1000.0), 'unit': 'images/s', 'ms_per_call': e2e_ms,
                  'h2d_bytes_per_step': batch * SEP_N * SEP_N * 4, 'd2h_bytes_per_step': 2 * batch * SEP_N * SEP_N * 4}
    if cpu_sample and rank == 0:
        from oracle import rwt
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        rwt.separate(host[0].astype(np.float64), SEP_DCOMP, SEP_DSIZE, nthreads=cores, **SEP_ARGS)
        dt = time.perf_counter() - t0
        out['cpu_baseline'] = {'value': 1.0 / dt, 'unit': 'images/s', 'cores': cores, 'kind': 'port',
                               'sample': 'one 256x256 image through the FP64 oracle of separate.m (%.1f s)' % dt}
    plan.close()
    return out


def run_gpu(args):
    import torch
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image, uneven_batch, BATCH_SIZES

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    stream = torch.cuda.current_stream()

    plan = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, batch=BATCH)
    scal = sc.nsst_scalars(plan, seed=100)  # product's Monte-Carlo scalars (setup, untimed)
    # the directional kernels: the autotuner's pick for this batch (setup,
    # untimed), or the one forced on the command line
    tune = None
    if args.directional == 'auto':
        tune = plan.autotune(BATCH)
    elif args.directional in ('split', 'fused'):
        plan.set_directional(args.directional)
    else:
        names = plan.directional_candidates()
        if args.directional not in names:
            raise SystemExit('--directional: %r is none of auto, split, fused, %s' % (args.directional, ', '.join(names)))
        plan.select_directional(BATCH, names.index(args.directional))
    plan.use_graphs(True)
    host = []
    for i in range(BATCH):
        _, noisy = noisy_image(H, W, SIGMA, 1000 * rank + i)
        host.append(noisy.astype(np.float32))
    xs = [torch.tensor(h, device=dev) for h in host]
    outs = [torch.empty_like(x) for x in xs]
    sig = [SIGMA] * BATCH
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        sc.nsst_denoise_batch(xs, plan, sig, K, None, outs=outs)

    # kernels per step: one eager pass counted by the library
    plan.use_graphs(False)
    c0 = sc.launch_count()
    step()
    kernels_per_step = sc.launch_count() - c0
    plan.use_graphs(True)
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    times = []
    for _ in range(args.steps):
        flush.fill_(1.0)  # evict L2 between timed steps (256 MB > 129 MB L2)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        times.append((e0, e1))
    barrier()
    clocks = sampler.stop()
    total_ms = sum(a.elapsed_time(b) for a, b in times)
    total_ms = max_over_ranks(total_ms, dev)
    ms_per_step = total_ms / args.steps
    value = job_throughput(BATCH * args.steps, world, total_ms / 1000.0)

    # ---- per-stage timing of the same batched pass (eager, events per stage)
    plan.use_graphs(False)
    plan.enable_timers(True)
    stage_ms = {}
    for _ in range(3):
        flush.fill_(1.0)
        step()
        for name, ms in plan.read_timers():
            stage_ms.setdefault(name, []).append(ms)
    plan.enable_timers(False)
    plan.use_graphs(True)
    stage_avg = {k: float(np.median(v)) for k, v in stage_ms.items()}
    peak, peak_kind = measured_peak()
    traffic_db = None
    tpath = os.path.join(ROOT, 'profiles', 'ncu_traffic.json')
    if os.path.exists(tpath) and (H, W) == (512, 512):  # captured at 512x512
        try:
            traffic_db = json.load(open(tpath))
        except ValueError:
            traffic_db = None
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    roofline = roofline_report(stage_avg, BATCH, H, W, peak, peak_kind, ms_per_step, sms, traffic_db)
    # the split kernels' own bytes (band planes materialised), for the dominant one
    dom = max(stage_avg, key=stage_avg.get)
    mat = algorithmic_bytes(dom, BATCH, H, W)
    if mat:
        roofline['dominant_launch'] = {'kernel': dom, 'ms': stage_avg[dom], 'bytes_as_designed': mat,
                                       'achieved_gbs': mat / (stage_avg[dom] / 1000.0) / 1e9}

    metric = METRIC if (H, W) == (512, 512) else METRIC.replace('512^2', '%dx%d' % (H, W))
    line = {'metric': metric, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': ms_per_step, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic (seeded ellipses + gradient + N(0, 20^2))',
            'config': {'workload': 'batch of %d x %dx%d images, one batched NSST dec+hard-thresh+rec pass per step'
                                   % (BATCH, H, W),
                       'H': H, 'W': W, 'batch_per_gpu': BATCH, 'dcomp': DCOMP, 'dsize': DSIZE, 'lpfilt': 'maxflat',
                       'K': K, 'sigma': SIGMA, 'parallelism': 'replicas' if world > 1 else 'single',
                       'l2': 'flushed between steps (256 MB write, untimed)', 'graphs': True,
                       'pyramid': 'spectral (2-D DCT-II domain, NSST_PYRAMID_AUTO)',
                       'directional': tune['chosen'] if tune else args.directional},
            'gpu_launches': kernels_per_step * args.steps, 'kernels_per_step': kernels_per_step,
            'clocks': clocks, 'roofline': roofline}
    if tune:
        line['autotune'] = {'n': tune['n'], 'chosen': tune['chosen'],
                            'candidates_ms': {c: m for c, m in tune['candidates']},
                            'direct_support_px': tune['direct_support'], 'direct_err': tune['direct_err'],
                            'direct_bound_ms': tune['direct_bound_ms'], 'direct_wins': tune['direct_wins']}

    if not args.no_extras:
        # ---- e2e through the public API with host buffers: every step copies its
        # 64 images in from pinned host memory and its 64 results back; three
        # device buffer sets and two copy streams let step k+1's input copy and
        # step k-1's output copy run while step k is denoised (with two sets the
        # copies measured serialised with the compute: 5.40 against 5.09 ms).
        # Steps alternate between two different input sets, so the check after
        # the loop sees that each step's results came from its own inputs.
        NBUF = 3
        host_b = [noisy_image(H, W, SIGMA, 1000 * rank + BATCH + i)[1].astype(np.float32) for i in range(BATCH)]
        pin_in = [torch.from_numpy(np.stack(host)).pin_memory(), torch.from_numpy(np.stack(host_b)).pin_memory()]
        pin_out = [torch.empty((BATCH, H, W), dtype=torch.float32).pin_memory() for _ in range(NBUF)]
        dev_in = [torch.empty((BATCH, H, W), dtype=torch.float32, device=dev) for _ in range(NBUF)]
        dev_out = [torch.empty((BATCH, H, W), dtype=torch.float32, device=dev) for _ in range(NBUF)]
        views_in = [list(d.unbind(0)) for d in dev_in]
        views_out = [list(d.unbind(0)) for d in dev_out]
        s_h2d, s_d2h = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
        ev_h2d = [torch.cuda.Event() for _ in range(NBUF)]
        ev_comp = [torch.cuda.Event() for _ in range(NBUF)]
        ev_d2h = [torch.cuda.Event() for _ in range(NBUF)]

        def e2e_run(nsteps):
            for k in range(nsteps):
                b = k % NBUF
                if k >= NBUF:
                    s_h2d.wait_event(ev_comp[b])  # step k-NBUF has consumed dev_in[b]
                with torch.cuda.stream(s_h2d):
                    dev_in[b].copy_(pin_in[k % 2], non_blocking=True)
                    ev_h2d[b].record(s_h2d)
                stream.wait_event(ev_h2d[b])
                if k >= NBUF:
                    stream.wait_event(ev_d2h[b])  # step k-NBUF's results have left dev_out[b]
                sc.nsst_denoise_batch(views_in[b], plan, sig, K, None, outs=views_out[b])
                ev_comp[b].record(stream)
                s_d2h.wait_event(ev_comp[b])
                with torch.cuda.stream(s_d2h):
                    pin_out[b].copy_(dev_out[b], non_blocking=True)
                    ev_d2h[b].record(s_d2h)
            for b in range(min(NBUF, nsteps)):
                stream.wait_event(ev_d2h[(nsteps - 1 - b) % NBUF])

        e2e_run(3)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ne = max(4, args.steps // 2)
        # the host copies share the host's memory with whatever else the
        # machine runs: the median of three timed runs of ne steps
        runs = []
        for _ in range(3):
            e0.record(stream)
            e2e_run(ne)
            e1.record(stream)
            torch.cuda.synchronize()
            runs.append(e0.elapsed_time(e1) / ne)
        e2e_ms = sorted(runs)[1]
        # the host copies of the last NBUF steps' results (both input sets) are
        # the device path's outputs for those inputs, bit for bit
        xb = [torch.tensor(h, device=dev) for h in host_b]
        outs_b = sc.nsst_denoise_batch(xb, plan, sig, K, None)
        torch.cuda.synchronize()
        ref = [outs, outs_b]
        same = all(torch.equal(pin_out[k % NBUF][i], ref[k % 2][i].cpu())
                   for k in range(ne - NBUF, ne) for i in range(BATCH))
        line['e2e'] = {'value': BATCH * world / (e2e_ms / 1000.0), 'unit': UNIT,
                       'h2d_bytes_per_step': BATCH * H * W * 4, 'd2h_bytes_per_step': BATCH * H * W * 4,
                       'ms_per_step': e2e_ms, 'ms_per_step_runs': runs,
                       'pipelined': 'H2D / denoise / D2H of adjacent steps overlap',
                       'results_equal_device_path': same}

        # ---- plain path: one image per call through a single-image plan
        p1 = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W)
        p1.set_scalars(scal)
        o1 = torch.empty_like(xs[0])
        for _ in range(3):
            sc.nsst_denoise(xs[0], p1, SIGMA, K, None, out=o1)
        torch.cuda.synchronize()
        e0.record(stream)
        for i in range(BATCH):
            sc.nsst_denoise(xs[i], p1, SIGMA, K, None, out=o1)
        e1.record(stream)
        torch.cuda.synchronize()
        plain = BATCH / (e0.elapsed_time(e1) / 1000.0)
        line['plain_images_per_s'] = plain
        line['batched_vs_plain'] = value / world / plain

        # ---- uneven batch of 64 (sizes from the batched config), one captured graph
        items = uneven_batch(BATCH, seed=3, sizes=BATCH_SIZES)
        counts = {}
        for _, nz, _ in items:
            counts[nz.shape] = counts.get(nz.shape, 0) + 1
        plans, singles, uchoice = [], {}, {}
        for shp, cnt in counts.items():
            pp = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, shp[0], shp[1], batch=cnt)
            us = sc.nsst_scalars(pp, seed=100)
            uchoice['%dx%d' % shp] = pp.autotune(cnt)['chosen']
            plans.append(pp)
            p1s = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, shp[0], shp[1])
            p1s.set_scalars(us)
            p1s.autotune(1)
            p1s.use_graphs(True)
            singles[shp] = p1s
        m = sc.MultiBatch(plans)
        uxs = [torch.tensor(nz.astype(np.float32), device=dev) for _, nz, _ in items]
        uouts = [torch.empty_like(x) for x in uxs]
        usig = [s for _, _, s in items]
        for _ in range(3):
            m.denoise(uxs, usig, K, outs=uouts)
        torch.cuda.synchronize()
        nu = max(3, args.steps // 2)
        ut = 0.0
        for _ in range(nu):
            flush.fill_(1.0)
            e0.record(stream)
            m.denoise(uxs, usig, K, outs=uouts)
            e1.record(stream)
            torch.cuda.synchronize()
            ut += e0.elapsed_time(e1)
        npx = sum(x.numel() for x in uxs)
        # the plain path on the same 64 images: one call per image through a
        # single-image plan of its size (graph replay, tuned for one image)
        pouts = [torch.empty_like(x) for x in uxs]
        for _ in range(2):
            for x, o, sg in zip(uxs, pouts, usig):
                sc.nsst_denoise(x, singles[tuple(x.shape)], sg, K, None, out=o)
        torch.cuda.synchronize()
        pt = 0.0
        for _ in range(3):
            flush.fill_(1.0)
            e0.record(stream)
            for x, o, sg in zip(uxs, pouts, usig):
                sc.nsst_denoise(x, singles[tuple(x.shape)], sg, K, None, out=o)
            e1.record(stream)
            torch.cuda.synchronize()
            pt += e0.elapsed_time(e1)
        pt /= 3
        # the two paths may run different (tuned) kernels: the same math in a
        # different FP32 rounding order
        udiff = max(float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)) for a, b in zip(uouts, pouts))
        # each size's batch on its own (its plan, its images, one call): the sum
        # is what the graph's per-size branches cost back to back
        alone = {}
        for pp, shp in zip(plans, counts):
            sel = [i for i, x in enumerate(uxs) if tuple(x.shape) == shp]
            bx, bo, bs = [uxs[i] for i in sel], [uouts[i] for i in sel], [usig[i] for i in sel]
            for _ in range(2):
                sc.nsst_denoise_batch(bx, pp, bs, K, None, outs=bo)
            torch.cuda.synchronize()
            at = 0.0
            for _ in range(3):
                flush.fill_(1.0)
                e0.record(stream)
                sc.nsst_denoise_batch(bx, pp, bs, K, None, outs=bo)
                e1.record(stream)
                torch.cuda.synchronize()
                at += e0.elapsed_time(e1)
            alone['%dx%d' % shp] = at / 3
        ub = BATCH / (ut / nu / 1000.0)
        up = BATCH / (pt / 1000.0)
        line['uneven_b64'] = {'images_per_s': ub, 'ms_per_batch': ut / nu, 'megapixels': npx / 1e6,
                              'gigapixels_per_s': npx / (ut / nu / 1000.0) / 1e9,
                              'plain_images_per_s': up, 'plain_ms': pt, 'vs_plain': ub / up,
                              'plain_vs_batched_max_rel_l2': udiff, 'directional': uchoice,
                              'sizes_alone_ms': alone, 'sum_of_sizes_alone_ms': sum(alone.values()),
                              'sizes': {'%dx%d' % k: v for k, v in counts.items()}}
        m.close()
        del plans, singles

        # ---- single images at 1024^2 and 2048^2 (the plain pipeline as a
        # drop-in): images/s and per-stage times against the roofline
        big = {}
        for (Hb, Wb), seed in (((1024, 1024), 1), ((2048, 2048), 2)):
            pb = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, Hb, Wb)
            sc.nsst_scalars(pb, seed=100)
            tb = pb.autotune(1)
            xb = torch.tensor(noisy_image(Hb, Wb, SIGMA, seed)[1].astype(np.float32), device=dev)
            ob = torch.empty_like(xb)
            pb.use_graphs(True)
            for _ in range(3):
                sc.nsst_denoise(xb, pb, SIGMA, K, None, out=ob)
            torch.cuda.synchronize()
            reps = 10
            bt = 0.0
            for _ in range(reps):
                flush.fill_(1.0)
                e0.record(stream)
                sc.nsst_denoise(xb, pb, SIGMA, K, None, out=ob)
                e1.record(stream)
                torch.cuda.synchronize()
                bt += e0.elapsed_time(e1)
            bt /= reps
            pb.use_graphs(False)
            pb.enable_timers(True)
            st_ms = {}
            for _ in range(3):
                flush.fill_(1.0)
                sc.nsst_denoise(xb, pb, SIGMA, K, None, out=ob)
                for name, ms in pb.read_timers():
                    st_ms.setdefault(name, []).append(ms)
            pb.enable_timers(False)
            st_avg = {k: float(np.median(v)) for k, v in st_ms.items()}
            rf = roofline_report(st_avg, 1, Hb, Wb, peak, peak_kind, bt, sms, None)
            big['%dx%d' % (Hb, Wb)] = {'images_per_s': 1000.0 / bt, 'ms_per_image': bt,
                                        'directional': tb['chosen'], 'stages_ms': st_avg,
                                        'stage_groups': rf['stage_groups'], 'step': rf['step'],
                                        'compute': rf['compute']}
            del pb, xb, ob
            torch.cuda.empty_cache()
        line['single_image_p1k_p2k'] = big

        # ---- differentiable config: 16 x 512^2, forward vs forward + hand-written adjoint
        pd = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, batch=16)
        sc.autograd.enable_grad(pd)
        sd = sc.nsst_scalars(pd, seed=100)
        lv = pd.band_levels
        tau = torch.tensor([3.0 * SIGMA * sd[b] for b in range(pd.nbands)], dtype=torch.float32, device=dev)
        xd = torch.stack(xs[:16]).contiguous()
        cd = torch.stack([torch.tensor(noisy_image(H, W, 0.0, 1000 * rank + i)[0].astype(np.float32), device=dev)
                          for i in range(16)])
        def fwd():
            with torch.no_grad():
                return sc.nsst_denoise_diff(xd, tau, pd)
        def fwd_bwd():
            xg = xd.clone().requires_grad_(True)
            tg = tau.clone().requires_grad_(True)
            loss = torch.sum((sc.nsst_denoise_diff(xg, tg, pd) - cd) ** 2)
            loss.backward()
            return xg.grad, tg.grad
        for f in (fwd, fwd_bwd):
            for _ in range(3):
                f()
        torch.cuda.synchronize()
        res = {}
        for name, f in (('forward_ms', fwd), ('forward_adjoint_ms', fwd_bwd)):
            tt = 0.0
            for _ in range(5):
                flush.fill_(1.0)
                e0.record(stream)
                f()
                e1.record(stream)
                torch.cuda.synchronize()
                tt += e0.elapsed_time(e1)
            res[name] = tt / 5
        res['ratio'] = res['forward_adjoint_ms'] / res['forward_ms']
        res['images'] = 16
        line['differentiable_d16'] = res
        del pd

        # ---- 3-D volumes: batches of 4 x 128^3 and 4 x 192^3 (72 directional
        # bands, numDir 2, 2, 4), hard threshold, forward vs forward + adjoint
        line['volume_v3'] = volume_bench(sc, torch, dev, stream, flush, rank)

        # ---- image separation (points / curves), the demo's configuration, batch of 8
        line['separation'] = separation_bench(sc, torch, dev, stream, flush, rank, batch=args.sep_batch)

    if rank == 0:
        cb = cpu_baseline()
        line['cpu_baseline'] = cb
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


def run_v3(args):
    import torch
    import shearcuda_gb300 as sc
    dev = torch.device('cuda', 0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    sizes = tuple(int(v) for v in args.v3_sizes.split(','))
    res = volume_bench(sc, torch, dev, torch.cuda.current_stream(), flush, 0, reps=max(1, args.steps), sizes=sizes,
                       batch=args.v3_batch)
    print(json.dumps({'workload': 'v3', 'volume_v3': res}), flush=True)


def run_sep(args):
    import torch
    import shearcuda_gb300 as sc
    dev = torch.device('cuda', 0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    res = separation_bench(sc, torch, dev, torch.cuda.current_stream(), flush, 0, reps=max(1, args.steps),
                           batch=args.sep_batch, cpu_sample=False)
    print(json.dumps({'workload': 'sep', 'separation': res}), flush=True)


def main():
    args = parse()
    global BATCH, H, W
    BATCH = args.batch
    if args.impl == 'gb300' and args.workload == '2d' and not args.cpu_sweep:
        H, W = (int(v) for v in args.size.lower().split('x'))
    if args.cpu_sweep:
        cpu_sweep()
    elif args.impl == 'reference':
        run_reference(args)
    elif args.workload == 'v3':
        run_v3(args)
    elif args.workload == 'sep':
        run_sep(args)
    else:
        run_gpu(args)


if __name__ == '__main__':
    main()
