"""Seeded synthetic volumes for the smart-interpolation workloads.

No public dataset belongs to this path, so the benchmark inputs are drawn
from numpy.random.default_rng(seed):
  * ``plain_volume``   128^3 uint8: background mean 60 plus two ellipsoids
    (means 130 and 200, semi-axes U[15, 45]), N(0, 15) noise clipped to
    [0, 255]; labels 0..2 on every 10th z-slice;
  * ``allaxis_volume`` (400, 512, 512) uint8: 8 ellipsoid/tube phases with
    means spread over 30..230, N(0, 12) noise, 3-voxel Gaussian blur at the
    interfaces; labels 0..8 on every 8th XY slice and every 16th YZ / XZ slice;
  * ``batch_volumes``  uneven uint16 volumes (64^3 .. 384x320x256) with 2..12
    phases and label spacing 4..20;
  * ``large_volume``   1024^3 uint8 with 6 phases, uint8 labels on every 12th
    XY slice.
  * ``screw_like_volume`` 419x492x462 uint8 with 2 objects labelled every 20th
    z-slice (the dimensions and labelling of the reference's published
    "biological screw" timing; synthetic content).
Each generator returns (image, sparse labels, ground truth).
"""
from __future__ import annotations

import numpy as np


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d],
    ])


def _paint_ellipsoid(truth, label, center, semi, rot):
    Z, Y, X = truth.shape
    r = float(max(semi))
    lo = [max(0, int(np.floor(center[i] - r))) for i in range(3)]
    hi = [min(s, int(np.ceil(center[i] + r)) + 1) for i, s in enumerate((Z, Y, X))]
    if any(h <= l for l, h in zip(lo, hi)):
        return
    zz, yy, xx = np.meshgrid(*(np.arange(l, h, dtype=np.float32) - c for l, h, c in zip(lo, hi, center)),
                             indexing="ij")
    p = np.stack([zz, yy, xx], -1) @ rot.astype(np.float32)
    m = ((p / np.asarray(semi, np.float32)) ** 2).sum(-1) <= 1.0
    truth[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]][m] = label


def _paint_tube(truth, label, p0, p1, radius):
    Z, Y, X = truth.shape
    p0, p1 = np.asarray(p0, np.float32), np.asarray(p1, np.float32)
    lo = [max(0, int(np.floor(min(p0[i], p1[i]) - radius))) for i in range(3)]
    hi = [min(s, int(np.ceil(max(p0[i], p1[i]) + radius)) + 1) for i, s in enumerate((Z, Y, X))]
    if any(h <= l for l, h in zip(lo, hi)):
        return
    zz, yy, xx = np.meshgrid(*(np.arange(l, h, dtype=np.float32) for l, h in zip(lo, hi)), indexing="ij")
    p = np.stack([zz, yy, xx], -1)
    d = p1 - p0
    t = np.clip(((p - p0) @ d) / float(d @ d), 0.0, 1.0)
    dist2 = ((p - (p0 + t[..., None] * d)) ** 2).sum(-1)
    truth[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]][dist2 <= radius * radius] = label


def _render(truth, means, bg_mean, sigma, rng, blur=0.0, out_dtype=np.uint8, scale=1.0):
    lut = np.asarray([bg_mean] + list(means), np.float32)
    img = lut[truth]
    if blur > 0:
        from scipy.ndimage import gaussian_filter

        img = gaussian_filter(img, blur, mode="nearest", truncate=2.0)
    img += rng.normal(0.0, sigma, size=truth.shape).astype(np.float32)
    img *= np.float32(scale)
    hi = 255.0 * scale if out_dtype == np.uint8 else float(np.iinfo(out_dtype).max)
    np.clip(img, 0.0, hi, out=img)
    return np.rint(img).astype(out_dtype)


def sparse_labels(truth, z_every=None, y_every=None, x_every=None, dtype=np.int32):
    """Keeps the ground-truth labels on every n-th slice of each given axis."""
    lab = np.zeros(truth.shape, dtype)
    if z_every:
        lab[::z_every] = truth[::z_every]
    if y_every:
        lab[:, ::y_every] = truth[:, ::y_every]
    if x_every:
        lab[:, :, ::x_every] = truth[:, :, ::x_every]
    return lab


def plain_volume(seed=0, shape=(128, 128, 128), z_every=10, semi=(15, 45)):
    """Plain single-volume case (128^3 uint8, 2 ellipsoids, labels every 10th z)."""
    rng = np.random.default_rng(seed)
    truth = np.zeros(shape, np.uint8)
    for lab, _mean in ((1, 130), (2, 200)):
        s = rng.uniform(semi[0], semi[1], 3)
        c = [rng.uniform(0.3 * n, 0.7 * n) for n in shape]
        _paint_ellipsoid(truth, lab, c, s, _rotation(rng))
    img = _render(truth, (130, 200), 60, 15.0, rng)
    return img, sparse_labels(truth, z_every=z_every), truth


def _phases(rng, truth, n_phases, size_frac=(0.08, 0.25)):
    Z, Y, X = truth.shape
    n = min(Z, Y, X)
    for lab in range(1, n_phases + 1):
        if rng.random() < 0.6:
            s = rng.uniform(size_frac[0] * n, size_frac[1] * n, 3)
            c = [rng.uniform(0.15 * d, 0.85 * d) for d in (Z, Y, X)]
            _paint_ellipsoid(truth, lab, c, s, _rotation(rng))
        else:
            p0 = [rng.uniform(0.1 * d, 0.9 * d) for d in (Z, Y, X)]
            p1 = [rng.uniform(0.1 * d, 0.9 * d) for d in (Z, Y, X)]
            _paint_tube(truth, lab, p0, p1, rng.uniform(0.03 * n, 0.08 * n))


def allaxis_volume(seed=0, shape=(400, 512, 512), n_phases=8, z_every=8, yx_every=16):
    """All-axis case: (z, y, x) = (400, 512, 512), 8 phases, labels on every 8th
    XY slice plus every 16th YZ and XZ slice."""
    rng = np.random.default_rng(seed)
    truth = np.zeros(shape, np.uint8)
    _phases(rng, truth, n_phases)
    means = np.linspace(30, 230, n_phases).tolist()
    img = _render(truth, means, 10, 12.0, rng, blur=3.0)
    return img, sparse_labels(truth, z_every=z_every, y_every=yx_every, x_every=yx_every), truth


def batch_volumes(seed=0, count=32, lo=(64, 64, 64), hi=(256, 320, 384)):
    """Uneven uint16 volumes (z, y, x between 64^3 and 256x320x384) with 2..12
    phases and z-slice label spacing 4..20; returns a list of (img, labels, truth)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        shape = tuple(int(rng.integers(a, b + 1)) for a, b in zip(lo, hi))
        n_ph = int(rng.integers(2, 13))
        truth = np.zeros(shape, np.uint8)
        _phases(rng, truth, n_ph, size_frac=(0.1, 0.3))
        means = rng.uniform(20, 235, n_ph).tolist()
        img = _render(truth, means, 10, 10.0, rng, out_dtype=np.uint16, scale=200.0)
        every = int(rng.integers(4, 21))
        out.append((img, sparse_labels(truth, z_every=every), truth))
    return out


def large_volume(seed=0, shape=(1024, 1024, 1024), n_phases=6, z_every=12, slab=64):
    """Large case: 1024^3 uint8, 6 phases, labels on every 12th XY slice.
    Rendered in z-slabs to bound host memory."""
    rng = np.random.default_rng(seed)
    truth = np.zeros(shape, np.uint8)
    _phases(rng, truth, n_phases, size_frac=(0.1, 0.3))
    means = np.linspace(40, 220, n_phases).tolist()
    lut = np.asarray([10] + list(means), np.float32)
    img = np.empty(shape, np.uint8)
    for z0 in range(0, shape[0], slab):
        t = truth[z0:z0 + slab]
        v = lut[t]
        v += rng.normal(0.0, 12.0, size=t.shape).astype(np.float32)
        np.clip(v, 0.0, 255.0, out=v)
        img[z0:z0 + slab] = np.rint(v).astype(np.uint8)
    return img, sparse_labels(truth, z_every=z_every, dtype=np.uint8), truth


def _paint_shell(truth, label, center, semi, thickness, rot):
    """An ellipsoidal shell: the ellipsoid minus a smaller concentric one."""
    tmp = np.zeros_like(truth, dtype=bool)
    inner = [max(s - thickness, 1.0) for s in semi]
    t = np.zeros(truth.shape, np.uint8)
    _paint_ellipsoid(t, 1, center, semi, rot)
    _paint_ellipsoid(t, 2, center, inner, rot)
    tmp[t == 1] = True
    truth[tmp] = label


def smooth_noise(rng, shape, octaves=3, base=8):
    """Multi-octave smooth noise in [-1, 1] (sum of upsampled random lattices,
    each octave twice as fine and half as strong)."""
    from scipy.ndimage import zoom

    out = np.zeros(shape, np.float32)
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = [max(2, s // (base >> o) if (base >> o) else s) for s in shape]
        lat = rng.uniform(-1, 1, cells).astype(np.float32)
        up = zoom(lat, [s / c for s, c in zip(shape, cells)], order=1)[: shape[0], : shape[1], : shape[2]]
        out[: up.shape[0], : up.shape[1], : up.shape[2]] += amp * up
        total += amp
        amp *= 0.5
    return out / total


def procedural_volume(rng, shape=(96, 96, 96)):
    """Training volume: 2-8 phases of random ellipsoids, tubes and shells,
    smooth multi-octave intensity modulation, Gaussian noise sigma 5-25, uint8;
    labels on every k-th z-slice, k in 6..14."""
    n_ph = int(rng.integers(2, 9))
    truth = np.zeros(shape, np.uint8)
    n = min(shape)
    for lab in range(1, n_ph + 1):
        kind = rng.random()
        if kind < 0.45:
            s = rng.uniform(0.1 * n, 0.3 * n, 3)
            c = [rng.uniform(0.15 * d, 0.85 * d) for d in shape]
            _paint_ellipsoid(truth, lab, c, s, _rotation(rng))
        elif kind < 0.75:
            p0 = [rng.uniform(0.05 * d, 0.95 * d) for d in shape]
            p1 = [rng.uniform(0.05 * d, 0.95 * d) for d in shape]
            _paint_tube(truth, lab, p0, p1, rng.uniform(0.03 * n, 0.1 * n))
        else:
            s = rng.uniform(0.15 * n, 0.35 * n, 3)
            c = [rng.uniform(0.25 * d, 0.75 * d) for d in shape]
            _paint_shell(truth, lab, c, s, rng.uniform(2.0, 0.1 * n), _rotation(rng))
    means = rng.uniform(20, 235, n_ph + 1).astype(np.float32)
    img = means[truth]
    img *= 1.0 + 0.25 * smooth_noise(rng, shape)
    img += rng.normal(0.0, rng.uniform(5, 25), size=shape).astype(np.float32)
    np.clip(img, 0, 255, out=img)
    every = int(rng.integers(6, 15))
    return np.rint(img).astype(np.uint8), sparse_labels(truth, z_every=every), truth


def screw_like_volume(seed=0, shape=(419, 492, 462), z_every=20):
    """Dimensions and labelling of the reference's published end-to-end timing
    case (419x492x462, 2 objects labelled on every 20th slice) with synthetic
    content: a tube (screw shaft) and an ellipsoid, noise sigma 12."""
    rng = np.random.default_rng(seed)
    truth = np.zeros(shape, np.uint8)
    Z, Y, X = shape
    _paint_tube(truth, 1, (0.1 * Z, 0.5 * Y, 0.45 * X), (0.9 * Z, 0.5 * Y, 0.55 * X), 0.15 * min(Y, X))
    _paint_ellipsoid(truth, 2, (0.5 * Z, 0.3 * Y, 0.7 * X), (0.2 * Z, 0.12 * Y, 0.12 * X), _rotation(rng))
    img = _render(truth, (150, 210), 40, 12.0, rng)
    return img, sparse_labels(truth, z_every=z_every), truth


def blob_volume(shape, seed, labels, centres, radii, noise, dtype=np.uint8, jitter=1.5):
    """Image of bright/dark ellipsoids with noise, and a label volume of the
    same ellipsoids with perturbed radii (a segmentation to be refined)."""
    rng = np.random.default_rng(seed)
    zz, yy, xx = np.meshgrid(*[np.arange(s, dtype=np.float64) for s in shape], indexing="ij")
    img = np.full(shape, 60.0)
    lab = np.zeros(shape, np.int32)
    for k, (lv, c, r) in enumerate(zip(labels, centres, radii)):
        d = ((zz - c[0]) / r[0]) ** 2 + ((yy - c[1]) / r[1]) ** 2 + ((xx - c[2]) / r[2]) ** 2
        img[d <= 1.0] = 110.0 + 50.0 * k
        rr = 1.0 + jitter * (rng.random(shape) - 0.5) / max(r)
        lab[d <= rr] = lv
    img += rng.normal(0.0, noise, shape)
    if dtype == np.uint8:
        img = np.clip(np.rint(img), 0, 255).astype(np.uint8)
    else:
        img = (img * 3.7 - 40.0).astype(dtype)
    return img, lab
