"""Seeded synthetic test images for the NSST denoising workloads.

No public dataset is involved: the reference demos use photographs that are
not shipped (shearcuda/test/deno_*_shearlets.m:17), so images are drawn from
a fixed generator: a linear intensity gradient, then 1-20 filled ellipses
(centre uniform over the image, semi-axes U[0.02, 0.3] * min(H, W), angle
U[0, pi), intensity U[0, 255]; later ellipses overwrite earlier ones), plus
i.i.d. N(0, sigma^2) noise.  All FP64 from numpy's PCG64 generator.
"""
import numpy as np

BATCH_SIZES = ((256, 256), (384, 512), (512, 512), (768, 1024), (1024, 1024))


def clean_image(H, W, rng):
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float64)
    u, v = yy / max(H - 1, 1), xx / max(W - 1, 1)
    theta = rng.uniform(0, 2 * np.pi)
    g0, g1 = rng.uniform(0, 128), rng.uniform(0, 96)
    img = g0 + g1 * (np.cos(theta) * u + np.sin(theta) * v)
    m = min(H, W)
    for _ in range(int(rng.integers(1, 21))):
        cy, cx = rng.uniform(0, H), rng.uniform(0, W)
        a, b = rng.uniform(0.02, 0.3, size=2) * m
        ang = rng.uniform(0, np.pi)
        val = rng.uniform(0, 255)
        c, s = np.cos(ang), np.sin(ang)
        dy, dx = yy - cy, xx - cx
        r1 = (c * dx + s * dy) / a
        r2 = (-s * dx + c * dy) / b
        img[r1 * r1 + r2 * r2 <= 1.0] = val
    return img


def noisy_image(H, W, sigma, seed):
    """(clean, noisy) FP64 pair for one seed."""
    rng = np.random.default_rng(seed)
    clean = clean_image(H, W, rng)
    noisy = clean + sigma * rng.standard_normal((H, W))
    return clean, noisy


def uneven_batch(n, seed, sizes=BATCH_SIZES, sigma_range=(10.0, 40.0)):
    """n (clean, noisy, sigma) triples with sizes drawn uniformly from `sizes`
    and sigma ~ U[sigma_range] per image."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        H, W = sizes[int(rng.integers(0, len(sizes)))]
        sigma = float(rng.uniform(*sigma_range))
        clean, noisy = noisy_image(H, W, sigma, seed * 100003 + i)
        out.append((clean, noisy, sigma))
    return out


def clean_volume(shape, rng, n_ellipsoids=None):
    """A sequence-like volume: 1-12 random ellipsoids (centre uniform,
    semi-axes U[0.05, 0.3] * min(shape), intensity U[0, 255]) whose centres
    move linearly along axis 2 (the time axis of a video volume) at a random
    velocity of up to 0.3 voxel per plane, over a constant background U[0, 64]."""
    n0, n1, n2 = shape
    x0 = np.arange(n0, dtype=np.float64)[:, None, None]
    x1 = np.arange(n1, dtype=np.float64)[None, :, None]
    t = np.arange(n2, dtype=np.float64)[None, None, :]
    vol = np.full(shape, rng.uniform(0, 64))
    m = min(shape)
    for _ in range(int(n_ellipsoids or rng.integers(1, 13))):
        c = rng.uniform(0, 1, size=3) * np.array(shape)
        ax = rng.uniform(0.05, 0.3, size=3) * m
        vel = rng.uniform(-0.3, 0.3, size=2)
        val = rng.uniform(0, 255)
        d0 = (x0 - c[0] - vel[0] * t) / ax[0]
        d1 = (x1 - c[1] - vel[1] * t) / ax[1]
        d2 = (t - c[2]) / ax[2]
        vol[d0 * d0 + d1 * d1 + d2 * d2 <= 1.0] = val
    return vol


def noisy_volume(shape, sigma, seed):
    """(clean, noisy) FP64 volume pair for one seed."""
    rng = np.random.default_rng(seed)
    clean = clean_volume(tuple(shape), rng)
    noisy = clean + sigma * rng.standard_normal(tuple(shape))
    return clean, noisy


def points_and_curves(N, npoints=150, sigma=20.0, seed=0, amp=255.0):
    """A square test image of side N for the points / curves separation: a
    smooth bump as background, straight lines of several slopes and a ring
    (all two pixels wide, value amp), npoints isolated one-pixel points (value
    amp), plus N(0, sigma^2) noise.  Returns (clean, noisy) float64.  The
    separation demo's own generator is of this kind (curves, points, noise)
    at N = 256 with 150 points and sigma 20."""
    rng = np.random.default_rng(seed)
    r, c = np.mgrid[0:N, 0:N].astype(np.float64) / N
    img = amp / (1.0 + np.hypot(r - 0.15, c - 0.1)) ** 3 * 0.8
    cols = np.arange(N)
    for _ in range(5):  # lines row = slope * col + offset, or transposed
        slope = rng.uniform(-2.5, 2.5)
        off = rng.uniform(0.1, 0.9) * N - slope * N / 2
        rows = np.round(slope * cols + off).astype(int)
        for d in (0, 1):
            ok = (rows + d >= 0) & (rows + d < N)
            if rng.random() < 0.5:
                img[rows[ok] + d, cols[ok]] = amp
            else:
                img[cols[ok], rows[ok] + d] = amp
    rad = np.hypot(r - 0.5, c - 0.5) * N
    ring = rng.uniform(0.25, 0.4) * N
    img[(rad > ring) & (rad < ring + 2.0)] = amp
    pts = rng.integers(0, N, size=(npoints, 2))
    img[pts[:, 0], pts[:, 1]] = amp
    return img, img + sigma * rng.standard_normal((N, N))
