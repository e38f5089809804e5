"""Command-line front end of the autotuner (nsst_plan_autotune).

    python -m shearcuda_gb300.tune [--sizes 512x512:64,256x256:64 ...]

For every H x W : n pair it builds a plan of batch capacity n (dcomp
[3 3 4 4], dsize [32 32 16 16], maxflat, Monte-Carlo scalars), tunes it for n
images and prints one JSON line: the candidates' median milliseconds for one
directional-stage pass, the chosen one, and the direct-convolution evaluation
(window per level, truncation error, lower bound).
"""
import argparse
import json

DEFAULT = ('512x512:64,512x512:8,512x512:1,256x256:64,256x256:8,256x256:1,384x512:32,384x512:1,'
           '1024x1024:8,1024x1024:1,768x1024:8,256x384:8')


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--sizes', default=DEFAULT, help='comma-separated HxW:n')
    ap.add_argument('--dcomp', default='3,3,4,4')
    ap.add_argument('--dsize', default='32,32,16,16')
    a = ap.parse_args(argv)
    import shearcuda_gb300 as sc
    dcomp = [int(v) for v in a.dcomp.split(',')]
    dsize = [int(v) for v in a.dsize.split(',')]
    for item in a.sizes.split(','):
        hw, n = item.split(':')
        H, W = (int(v) for v in hw.split('x'))
        n = int(n)
        plan = sc.prepare_shearing_filters_cuda(dcomp, dsize, H, W, batch=n)
        sc.nsst_scalars(plan, 100)
        r = plan.autotune(n)
        plan.check_device()
        print(json.dumps({'H': H, 'W': W, 'n': n, 'chosen': r['chosen'],
                          'candidates_ms': {c: round(m, 4) for c, m in r['candidates']},
                          'direct_support_px': r['direct_support'],
                          'direct_err': [float('%.3g' % e) for e in r['direct_err']],
                          'direct_bound_ms': round(r['direct_bound_ms'], 2), 'direct_wins': r['direct_wins']}),
              flush=True)
        plan.close()


if __name__ == '__main__':
    main()
