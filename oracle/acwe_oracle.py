"""Active-contour post-processing ('acwe' and 'refined') — CPU oracle, TEST
INFRASTRUCTURE ONLY.

Only ``tests/`` and the CPU-baseline leg of ``bench.py`` use this module; the
product (``biomedisa_gb300.active_contour``) never does. It restates, in
vectorised NumPy, biomedisa/features/active_contour.py:109-225
(``activeContour`` and ``refinement``) and curvop_numba.py:5-149
(``evolution``, ``erosion``, ``dilation``, ``curvop``) with numba's scalar
typing:
  * evolution: |mean[label] - img| in binary32 (float32 - uint8 is float32
    in numba), alpha * that in binary64 for label 0, comparisons in binary64;
  * erosion: the plane sums |start - label| in int64 (no uint8 wrap);
  * refinement's chamfer scan (active_contour.py:45-81) equals the geodesic
    raster scan with a zero image, lamb = 0 and one iteration (same 13
    neighbours and domain, cost c + d in binary64, binary32 store), so it is
    computed by ``geo_oracle.raster_scan`` — the literal sequential scan, the
    yardstick of the device's Jacobi band.
The refinement's per-slice statistics use NumPy's mean, std and exp on the
slice arrays exactly as the reference writes them.
Pinned by tests/golden/ref_acwe.npz, made by the reference's own functions
(tests/golden/make_golden_acwe.py).
"""
from __future__ import annotations

import numpy as np

import geo_oracle

# The 27 neighbour offsets in the reference's loop order (dz outer, dx inner).
OFFSETS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def _plane_members():
    """The nine 3x3 planes through the centre (curvop_numba.py:125-134) as lists
    of indices into OFFSETS: x = 0, y = 0, z = 0, y = x, y = -x, z = x,
    z = -x, z = y, z = -y (offset coordinates in -1..1)."""
    tests = [
        lambda z, y, x: x == 0, lambda z, y, x: y == 0, lambda z, y, x: z == 0,
        lambda z, y, x: y == x, lambda z, y, x: y == -x, lambda z, y, x: z == x,
        lambda z, y, x: z == -x, lambda z, y, x: z == y, lambda z, y, x: z == -y,
    ]
    return [[i for i, o in enumerate(OFFSETS) if t(*o)] for t in tests]


PLANES = _plane_members()


def img_to_uint8(img):
    """biomedisa_helper.py:345-352: non-uint8 input is shifted by its minimum,
    divided by the new maximum and scaled by 255 in binary32, then truncated."""
    img = np.asarray(img)
    if img.dtype == np.uint8:
        return img
    f = img.astype(np.float32)
    f -= np.amin(f)
    with np.errstate(invalid="ignore", divide="ignore"):
        f /= np.amax(f)
        f *= np.float32(255.0)
        return np.where(np.isfinite(f), f, 0).astype(np.uint8)


def all_labels_of(labels):
    """pre_processing's label list (biomedisa_helper.py:671-694): the sorted
    distinct values, with 0 first even where no voxel holds it."""
    v = np.unique(labels)
    return v if v.size and v[0] == 0 else np.concatenate([[0], v]).astype(v.dtype)


def crop_box(lab_padded):
    """reduce_blocksize (active_contour.py:84-104): the box of the nonzero
    labels grown by 100 voxels on each side, clamped, as half-open ranges
    (z0, z1, y0, y1, x0, x1) of the padded volume."""
    shape = lab_padded.shape
    nz = np.nonzero(lab_padded)
    box = []
    for a, s in enumerate(shape):
        lo, hi = (int(nz[a].min()), int(nz[a].max())) if nz[0].size else (s, 0)
        lo = lo - 100 if lo - 100 > 0 else 0
        hi = hi + 100 if hi + 100 < s else s
        box += [lo, hi]
    return tuple(box)


def _neighbours(a):
    """The 27 shifted views of a (offset order) over the interior voxels."""
    Z, Y, X = a.shape
    return [a[1 + dz:Z - 1 + dz, 1 + dy:Y - 1 + dy, 1 + dx:X - 1 + dx] for dz, dy, dx in OFFSETS]


def _interior(a):
    return a[1:-1, 1:-1, 1:-1]


def label_means(data, labels):
    """mean[k] = float32(np.mean(data[labels == k])) for the labels present,
    0 elsewhere (active_contour.py:191-195). The float64 mean of integers is
    their exact sum divided once."""
    mean = np.zeros(256, np.float32)
    lab = labels.astype(np.int64).ravel()
    cnt = np.bincount(lab, minlength=256)
    tot = np.bincount(lab, weights=data.ravel().astype(np.float64), minlength=256)
    for k in np.nonzero(cnt)[0]:
        mean[k] = np.float32(tot[k] / cnt[k])
    return mean


def evolution(mean, A, data, alpha):
    """curvop_numba.py:5-29: every interior voxel takes, among its own label and
    the differing labels of its 27 neighbours (scan order, strict <), the one
    whose mean is closest to its intensity; label 0's distance is scaled by
    alpha."""
    B = A.copy()
    if min(A.shape) < 3:
        return B
    img = _interior(data).astype(np.float32)
    alpha = np.float64(alpha)

    def cost(lab):
        d = np.abs(mean[lab] - img).astype(np.float64)
        return np.where(lab == 0, alpha * d, d)

    ref_lab = _interior(A).astype(np.int64)
    ref = cost(ref_lab)
    fin = ref_lab.copy()
    for nb in _neighbours(A):
        t = nb.astype(np.int64)
        val = cost(t)
        upd = (t != ref_lab) & (val < ref)
        ref = np.where(upd, val, ref)
        fin = np.where(upd, t, fin)
    _interior(B)[...] = fin
    return B


def erosion(start, label):
    """curvop_numba.py:31-60 (returns the new volume): an interior voxel of the
    label with a differing neighbour keeps the label when one of the nine
    planes through it is all label, else takes the last differing neighbour
    in scan order."""
    out = start.copy()
    if min(start.shape) < 3:
        return out
    nbs = [nb.astype(np.int64) for nb in _neighbours(start)]
    eq = [nb == label for nb in nbs]
    found = ~np.logical_and.reduce(eq)
    keep = np.zeros_like(found)
    for members in PLANES:
        keep |= np.logical_and.reduce([eq[i] for i in members])
    cond = (_interior(start) == label) & found & ~keep
    sub = np.full(found.shape, label, np.int64)
    for nb, e in zip(nbs, eq):
        sub = np.where(~e, nb, sub)
    core = _interior(out)
    core[...] = np.where(cond, sub, core).astype(out.dtype)
    return out


def dilation(start, label):
    """curvop_numba.py:62-84 (returns the new volume). Its plane test can never
    pass (every plane sum counts the 18 voxels outside the plane), so every
    interior non-label voxel with a label voxel among its 27 neighbours
    becomes label."""
    out = start.copy()
    if min(start.shape) < 3:
        return out
    found = np.logical_or.reduce([nb == label for nb in _neighbours(start)])
    cond = (_interior(start) != label) & found
    core = _interior(out)
    core[...] = np.where(cond, label, core).astype(out.dtype)
    return out


def curvop(start, steps, label):
    """curvop_numba.py:86-149: even steps erode then dilate, odd steps dilate
    then erode; each operation reads the whole previous volume."""
    a = start.copy()
    for k in range(steps):
        if k % 2 == 0:
            a = dilation(erosion(a, label), label)
        else:
            a = erosion(dilation(a, label), label)
    return a


def chamfer_band(lab):
    """refinement's distance (active_contour.py:206-211): 0 on labelled
    voxels, 100 elsewhere, one forward/backward chamfer scan (1, sqrt2,
    sqrt3), then 1 where the distance exceeds 10. Returns (distance, band)
    with band = distance <= 10."""
    dist = np.zeros(lab.shape, np.float32)
    dist[lab == 0] = 100
    geo_oracle.raster_scan(np.zeros(lab.shape, np.float32), dist, 0.0, 1)
    return dist, dist <= 10


def refinement(data, lab, all_labels, margins=False):
    """active_contour.py:204-225 on the cropped, padded volumes. For every
    nonzero label (in order) and every z-slice whose band holds both label and
    non-label voxels, the slice is overwritten with the label where the
    band's Gaussian likelihood of the label exceeds that of the rest.
    margins=True also returns, per voxel, |p1 - p2| / max(p1, p2) of the
    decision that produced it (inf where no decision was made)."""
    _, band = chamfer_band(lab)
    result = np.zeros_like(lab)
    margin = np.full(lab.shape, np.inf)
    for l in all_labels[1:]:
        for k in range(lab.shape[0]):
            img, mask, b = data[k], lab[k], band[k]
            sel1, sel2 = b & (mask == l), b & (mask != l)
            if not (sel1.any() and sel2.any()):
                continue
            m1, s1 = np.mean(img[sel1]), np.std(img[sel1])
            m2, s2 = np.mean(img[sel2]), np.std(img[sel2])
            s1, s2 = max(s1, 1), max(s2, 1)
            p1 = np.exp(-(img - m1) ** 2 / (2 * s1 ** 2)) / np.sqrt(2 * np.pi * s1 ** 2)
            p2 = np.exp(-(img - m2) ** 2 / (2 * s2 ** 2)) / np.sqrt(2 * np.pi * s2 ** 2)
            result[k] = np.logical_and(b, p1 > p2) * l
            with np.errstate(invalid="ignore", divide="ignore"):
                margin[k] = np.where(b, np.abs(p1 - p2) / np.maximum(p1, p2), np.inf)
    return (result, margin) if margins else result


def active_contour(data, labels, alpha=1.0, smooth=1, steps=3, simple=False, margins=False):
    """activeContour (active_contour.py:109-202) for an image and a uint8 (or
    non-negative integer, <= 255) label volume of one shape: 'acwe'
    (simple=False) or 'refined' (simple=True). Returns uint8 labels of the
    input shape (and the refinement margins, see ``refinement``)."""
    labels = np.asarray(labels)
    d8 = img_to_uint8(data)
    all_labels = all_labels_of(labels)
    pad = [(1, 1)] * 3
    D = np.pad(d8, pad)
    L = np.pad(labels, pad)
    z0, z1, y0, y1, x0, x1 = crop_box(L)
    D = np.ascontiguousarray(D[z0:z1, y0:y1, x0:x1])
    L = np.ascontiguousarray(L[z0:z1, y0:y1, x0:x1])
    margin = None
    if simple:
        L, margin = refinement(D, L, all_labels, margins=True)
    else:
        for _ in range(steps):
            mean = label_means(D, L)
            L = evolution(mean, L, D, alpha)
            for k in all_labels:
                L = curvop(L, smooth, int(k))
    final = np.zeros(tuple(s + 2 for s in labels.shape), np.uint8)
    final[z0:z1, y0:y1, x0:x1] = L
    final = np.ascontiguousarray(final[1:-1, 1:-1, 1:-1])
    if margins:
        full = np.full(tuple(s + 2 for s in labels.shape), np.inf)
        if margin is not None:
            full[z0:z1, y0:y1, x0:x1] = margin
        return final, full[1:-1, 1:-1, 1:-1]
    return final
