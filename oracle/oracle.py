"""CPU oracle for the smart-interpolation hot path — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module; the product (``biomedisa_gb300``) never
does. Everything here is a plain restatement of the reference's algorithm in
NumPy (plus the C walker in ``walk_oracle.c`` for speed), written to be read
line by line against the cited reference files.

Parity contract with the GPU product:
  * integer hit maps, seeds (positions/slots/axes/labels, bit patterns of the
    float variance and weight constant), argmax labels: bit-exact;
  * smoothed maps and uncertainty: bit-exact, because both sides evaluate the
    same sequence of IEEE binary32 operations (no contraction).
Against the reference's own kernels (compiled as C by ``ref_extract.py``) the
same oracle loop, switched to the reference's RNG and ``expf`` weights,
reproduces the reference hit maps bit for bit (see tests/test_oracle_pin.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_BUILD = HERE / "_build"
_LIB = _BUILD / "libsi_oracle.so"

F32 = np.float32
U32 = np.uint32
M32 = np.uint64(0xFFFFFFFF)

# ---------------------------------------------------------------------------
# Reference host logic (biomedisa/features/biomedisa_helper.py)
# ---------------------------------------------------------------------------


def unique(arr):
    """biomedisa_helper.py:82-103 — sorted unique values."""
    return np.unique(arr)


def pre_processing(labelData, only="all", ignore="none"):
    """biomedisa_helper.py:639-724 (label part). Returns (labelData, allLabels)
    or raises ValueError where the reference reports an error."""
    labelData = np.array(labelData, copy=True)
    if labelData.ndim != 3:
        raise ValueError("Label data must be three-dimensional.")
    if labelData.dtype in (np.float16, np.float32, np.float64):
        labelData = labelData.astype(np.int32)
    allLabels = unique(labelData)
    if np.any(allLabels < 0):
        allLabels = np.delete(allLabels, np.argwhere(allLabels < 0))
    if np.any(allLabels > 255):
        labelData[labelData > 255] = 0
        allLabels = np.delete(allLabels, np.argwhere(allLabels > 255))
    if not np.any(allLabels == 0):
        allLabels = np.append(0, allLabels)
    labels_to_compute = only.split(",")
    if not any(x in ["all", "All", "ALL"] for x in labels_to_compute):
        labels_to_remove = [k for k in allLabels if str(k) not in labels_to_compute and k > 0]
        for k in labels_to_remove:
            labelData[labelData == k] = 0
            allLabels = np.delete(allLabels, np.argwhere(allLabels == k))
    labels_to_remove = ignore.split(",")
    if not any(x in ["none", "None", "NONE"] for x in labels_to_remove):
        for k in labels_to_remove:
            try:
                k = int(k)
                labelData[labelData == k] = 0
                allLabels = np.delete(allLabels, np.argwhere(allLabels == k))
            except ValueError:
                pass
    if len(allLabels) < 2:
        raise ValueError("No labeled slices found.")
    return labelData, allLabels


def normalize_image(data):
    """biomedisa/interpolation.py:136-144: int8 -> uint8 (+128); other
    non-uint8 -> float32 scaled to [0, 255]."""
    if data.dtype == np.int8:
        return (data.astype(np.int16) + 128).astype(np.uint8)
    if data.dtype != np.uint8:
        d = data.astype(np.float32)
        d -= np.amin(d)
        d /= np.amax(d)
        d *= 255.0
        return d
    return data


def smooth_img_3x3(img):
    """biomedisa_helper.py:308-323 — box mean over in-bounds neighbours,
    float64 accumulation in (k, l, m) order; uint8 output truncates."""
    zsh, ysh, xsh = img.shape
    src = img.astype(np.float64)
    tot = np.zeros(img.shape, np.float64)
    cnt = np.zeros(img.shape, np.int64)
    for k in (-1, 0, 1):
        for l in (-1, 0, 1):
            for m in (-1, 0, 1):
                dz = slice(max(0, -k), zsh - max(0, k))
                dy = slice(max(0, -l), ysh - max(0, l))
                dx = slice(max(0, -m), xsh - max(0, m))
                sz = slice(max(0, k), zsh - max(0, -k))
                sy = slice(max(0, l), ysh - max(0, -l))
                sx = slice(max(0, m), xsh - max(0, -m))
                tot[dz, dy, dx] = tot[dz, dy, dx] + src[sz, sy, sx]
                cnt[dz, dy, dx] += 1
    res = tot / cnt
    if img.dtype == np.uint8:
        return res.astype(np.uint8)
    return res.astype(img.dtype)


def read_labeled_slices(arr):
    """biomedisa_helper.py:1015-1022."""
    idx = [k for k in range(arr.shape[0]) if np.any(arr[k])]
    return idx, arr[idx].astype(np.int32) if idx else np.zeros((0,) + arr.shape[1:], np.int32)


def _allx_ones(arr, positive=False):
    """The one-pixel-line removal of biomedisa_helper.py:1024-1037 (labels
    != 0; positive=True: labels > 0, as the large path's reader,
    :1082-1094)."""
    ones = ((arr > 0) if positive else (arr != 0)).astype(np.int8)
    grad = np.zeros(arr.shape, np.int8)
    tmp = np.abs(ones[:, :-1] - ones[:, 1:])
    grad[:, :-1] += tmp
    grad[:, 1:] += tmp
    ones[grad == 2] = 0
    grad.fill(0)
    tmp = np.abs(ones[:, :, :-1] - ones[:, :, 1:])
    grad[:, :, :-1] += tmp
    grad[:, :, 1:] += tmp
    ones[grad == 2] = 0
    return ones


def read_indices_allx(arr, ax):
    """biomedisa_helper.py:1047-1066."""
    ones = _allx_ones(arr)
    return [(k, ax) for k in range(arr.shape[0]) if np.any(ones[k])]


def read_labeled_slices_allx(arr, ax):
    """biomedisa_helper.py:1024-1045."""
    ones = _allx_ones(arr)
    idx = [k for k in range(arr.shape[0]) if np.any(ones[k])]
    data = arr[idx].astype(np.int32) if idx else np.zeros((0,) + arr.shape[1:], np.int32)
    return [(k, ax) for k in idx], data


def allaxis_indices(labelData):
    """Slice indices of the three axes as interpolation.py:162-173 builds them."""
    out = list(read_indices_allx(labelData, 0))
    tmp = np.ascontiguousarray(np.swapaxes(labelData, 0, 1))
    out += read_indices_allx(tmp, 1)
    tmp = np.ascontiguousarray(np.swapaxes(tmp, 0, 2))
    out += read_indices_allx(tmp, 2)
    return out


def slices_adjacent(indices):
    """interpolation.py:175-183: True if two labelled slices of one axis touch."""
    for k in range(3):
        sub = [x for (x, y) in indices if y == k]
        if any((i - 1) in sub for i in sub):
            return True
    return False


def predict_blocksize(labelData):
    """biomedisa_helper.py:1105-1124 -> (zmin, zmax, ymin, ymax, xmin, xmax)."""
    zsh, ysh, xsh = labelData.shape
    nz = np.nonzero(labelData)
    if len(nz[0]) == 0:
        az, bz, ay, by, ax, bx = zsh, 0, ysh, 0, xsh, 0
    else:
        az, bz = int(nz[0].min()), int(nz[0].max())
        ay, by = int(nz[1].min()), int(nz[1].max())
        ax, bx = int(nz[2].min()), int(nz[2].max())
    return (
        az - 100 if az - 100 > 0 else 0,
        bz + 100 if bz + 100 < zsh else zsh,
        ay - 100 if ay - 100 > 0 else 0,
        by + 100 if by + 100 < ysh else ysh,
        ax - 100 if ax - 100 > 0 else 0,
        bx + 100 if bx + 100 < xsh else xsh,
    )


def get_labels(pre_final, labels):
    """biomedisa_helper.py:1209-1213 (the smallest index present stays 0)."""
    final = np.zeros_like(pre_final)
    for k in unique(pre_final)[1:]:
        final[pre_final == k] = labels[k]
    return final


def dice_score(ground_truth, result):
    """biomedisa_helper.py:155-165 (average_dice=False)."""
    return 2 * np.logical_and(ground_truth == result, (ground_truth + result) > 0).sum() / float(
        (ground_truth > 0).sum() + (result > 0).sum()
    )


def label_dice(a, b, label):
    ma, mb = a == label, b == label
    den = ma.sum() + mb.sum()
    return 1.0 if den == 0 else 2.0 * np.logical_and(ma, mb).sum() / den


# ---------------------------------------------------------------------------
# Binary32 arithmetic helpers
# ---------------------------------------------------------------------------


def fmaf(a, b, c):
    """Correctly rounded binary32 fused multiply-add.

    Published method: S. Boldo, G. Melquiond, "Emulation of FMA and correctly
    rounded sums: proved algorithms using rounding to odd", IEEE TC 57(4), 2008.
    a*b is exact in binary64; the binary64 sum is rounded to odd (TwoSum error
    term + sticky adjustment); rounding that to binary32 is then exact because
    53 >= 24 + 2.
    """
    a = np.asarray(a, F32).astype(np.float64)
    b = np.asarray(b, F32).astype(np.float64)
    cd = np.asarray(c, F32).astype(np.float64)
    p = a * b
    s = p + cd
    bb = s - p
    e = (p - (s - bb)) + (cd - bb)
    odd = (np.asarray(s).view(np.int64) & 1) == 1
    adj = (e != 0) & ~odd
    s = np.where(adj, np.nextafter(s, np.where(e > 0, np.inf, -np.inf)), s)
    return s.astype(F32)


LOG2E = F32(1.44269502162933349609375)
MAGIC = F32(12582912.0)
P5, P4, P3, P2, P1 = (F32(0.0013260921696200967), F32(0.009670175611972809), F32(0.055507123470306396),
                      F32(0.2402222454547882), F32(0.6931470036506653))


def weight_constant(var):
    """c = RN(RN(1 / RN(2 var)) * log2e)."""
    var = np.asarray(var, F32)
    div1 = F32(1.0) / (F32(2.0) * var)
    return (div1 * LOG2E).astype(F32)


def edge_weight(d2, c):
    """w = 2^(-d2 c): exponent split + degree-5 polynomial (same method and
    coefficients as the product)."""
    d2 = np.asarray(d2, F32)
    c = np.asarray(c, F32)
    y = (d2 * c).astype(F32)
    r = (y + MAGIC).astype(F32)
    kf = (r - MAGIC).astype(F32)
    g = (kf - y).astype(F32)
    p = fmaf(P5, g, P4)
    p = fmaf(p, g, P3)
    p = fmaf(p, g, P2)
    p = fmaf(p, g, P1)
    p = fmaf(p, g, F32(1.0))
    k = r.view(np.int32).astype(np.int64) - 0x4B400000
    bits = (p.view(np.int32).astype(np.int64) - (k << 23)).astype(np.int32)
    w = bits.view(F32)
    return np.where(y < F32(125.0), w, F32(0.0)).astype(F32)


# ---------------------------------------------------------------------------
# Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)
# ---------------------------------------------------------------------------


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c0, c1, c2, c3 = (np.asarray(v, np.uint64) & M32 for v in (c0, c1, c2, c3))
    k0 = np.uint64(int(k0) & 0xFFFFFFFF)
    k1 = np.uint64(int(k1) & 0xFFFFFFFF)
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(0x9E3779B9)) & M32
            k1 = (k1 + np.uint64(0xBB67AE85)) & M32
        p0 = c0 * np.uint64(0xD2511F53)
        p1 = c2 * np.uint64(0xCD9E8D57)
        hi0, lo0 = p0 >> np.uint64(32), p0 & M32
        hi1, lo1 = p1 >> np.uint64(32), p1 & M32
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return tuple(v.astype(U32) for v in (c0, c1, c2, c3))


def philox_python(ctr, key):
    """Scalar Philox4x32-10 in plain Python integers (independent check)."""
    c = list(ctr)
    k0, k1 = key
    for r in range(10):
        if r:
            k0 = (k0 + 0x9E3779B9) & 0xFFFFFFFF
            k1 = (k1 + 0xBB67AE85) & 0xFFFFFFFF
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & 0xFFFFFFFF, p1 & 0xFFFFFFFF, ((p0 >> 32) ^ c[3] ^ k1) & 0xFFFFFFFF,
             p0 & 0xFFFFFFFF]
    return tuple(c)


def u01(bits):
    return ((np.asarray(bits, U32) >> U32(8)).astype(F32) * F32(5.9604644775390625e-8)).astype(F32)


# ---------------------------------------------------------------------------
# Seeds
# ---------------------------------------------------------------------------


@dataclass
class Seeds:
    pos: np.ndarray      # uint32 linear index in the working volume
    slot: np.ndarray     # uint32 label slot
    axis: np.ndarray     # uint32 seed axis
    label: np.ndarray    # uint32 label value
    b: np.ndarray        # float32 seed intensity
    var: np.ndarray      # float32 clamped variance
    rng_cuda: np.ndarray  # uint32 reference CUDA MRG init (slice-stack index)
    rng_ocl: np.ndarray   # uint32 reference OpenCL MRG init (global index)

    def __len__(self):
        return len(self.pos)

    @property
    def c(self):
        return weight_constant(self.var)


def read_labeled_slices_large(arr):
    """biomedisa_helper.py:1068-1080: z-slices with any non-zero label; after
    each one taken, the next four are skipped."""
    idx, i = [], 0
    while i < arr.shape[0]:
        if np.any(arr[i]):
            idx.append(i)
            i += 5
        else:
            i += 1
    return idx


def large_slice_box(stack):
    """pycuda_large.py:39-58 (reduceBlocksize) on the stack of taken slices:
    the in-plane box of the non-zero labels of slices whose non-zero voxels
    are not all in column 0, grown by 100 and clamped; returns (y0, y1, x0,
    x1) — the stack is -1 outside [y0, y1) x [x0, x1)."""
    zsh, ysh, xsh = stack.shape
    amin_x, amax_x, amin_y, amax_y = xsh, 0, ysh, 0
    for k in range(zsh):
        y, x = np.nonzero(stack[k])
        if x.any():
            amin_x = min(amin_x, int(np.amin(x)))
            amax_x = max(amax_x, int(np.amax(x)))
            amin_y = min(amin_y, int(np.amin(y)))
            amax_y = max(amax_y, int(np.amax(y)))
    amin_x = amin_x - 100 if amin_x - 100 > 0 else 0
    amax_x = amax_x + 100 if amax_x + 100 < xsh else xsh
    amin_y = amin_y - 100 if amin_y - 100 > 0 else 0
    amax_y = amax_y + 100 if amax_y + 100 < ysh else ysh
    return amin_y, amax_y, amin_x, amax_x


def read_labeled_slices_allx_large(arr):
    """biomedisa_helper.py:1082-1099: the slices keeping a positive label
    after the one-pixel-line removal (no slice skipping)."""
    ones = _allx_ones(arr, positive=True)
    return [k for k in range(arr.shape[0]) if np.any(ones[k])]


def large_allx_slice_list(lab):
    """The all-axis large path's slices (rw_large.py:68-107 on one GPU):
    (axis, index) for z-slices of the crop, then y- and x-slices read from the
    swapped crops."""
    t1 = np.ascontiguousarray(np.swapaxes(lab, 0, 1))
    t2 = np.ascontiguousarray(np.swapaxes(t1, 0, 2))
    return ([(0, k) for k in read_labeled_slices_allx_large(lab)] +
            [(1, k) for k in read_labeled_slices_allx_large(t1)] +
            [(2, k) for k in read_labeled_slices_allx_large(t2)])


def large_allx_labels(work_labels, slice_list):
    """Per axis, the cropped label volume as that axis' slice stack holds it
    after reduceBlocksize (pycuda_large_allx.py:37-57): the stack's box is
    taken over its labels other than 0 and -1 (slices whose such labels all
    sit in column 0 do not count), grown by 100 and clamped in the stack's
    (row, column) plane; the axis' slices read -1 outside it. Returns
    ({axis: volume}, {axis: (r0, r1, c0, c1)})."""
    vols, boxes = {}, {}
    for axis in (0, 1, 2):
        lab = np.array(work_labels, dtype=np.int32, copy=True)
        idx = [k for a, k in slice_list if a == axis]
        if idx:
            stack = np.stack([_slice_view(lab, axis, k) for k in idx])
            stack[stack == -1] = 0
            r0, r1, c0, c1 = large_slice_box(stack)
            for k in idx:
                view = _slice_view(lab, axis, k)
                view[:r0] = -1
                view[r1:] = -1
                view[:, :c0] = -1
                view[:, c1:] = -1
            boxes[axis] = (r0, r1, c0, c1)
        vols[axis] = lab
    return vols, boxes


def _window_count(mask, r, c):
    """For each (r[i], c[i]): the number of True entries of the 2-D mask in
    rows max(1, r-100)..min(R-2, r+100) and columns max(1, c-100)..min(C-2,
    c+100) (the adaptive window clipped to the plane's interior), from an
    integral image."""
    R, C = mask.shape
    ii = np.zeros((R + 1, C + 1), np.int64)
    ii[1:, 1:] = mask.astype(np.int64).cumsum(0).cumsum(1)
    r0, r1 = np.maximum(1, r - 100), np.minimum(R - 2, r + 100) + 1
    c0, c1 = np.maximum(1, c - 100), np.minimum(C - 2, c + 100) + 1
    return ii[r1, c1] - ii[r0, c1] - ii[r1, c0] + ii[r0, c0]


def _adaptive_keep(plane, r, c, own):
    """Seeds at (r, c) of one slice plane with labels own: kept iff
    (r + c) % 4 == 0 or the window holds a label other than own and -1
    (count of non-(-1) labels minus count of own labels > 0)."""
    keep = (r + c) % 4 == 0
    other = _window_count(plane != -1, r, c)
    for v in np.unique(own):
        sel = own == v
        other[sel] -= _window_count(plane == v, r[sel], c[sel])
    return keep | (other > 0)


def adaptive_seed_mask_allx(large_labs, seeds):
    """The all-axis large walker's adaptive test (pycuda_large_allx.py:513-533
    and :683-703): as adaptive_seed_mask, in the (row, column) plane of the
    seed's own slice (z-slices (y, x), y-slices (z, x), x-slices (z, y)),
    with that axis' labels."""
    keep = np.zeros(len(seeds), bool)
    if not len(seeds):
        return keep
    Z, Y, X = next(iter(large_labs.values())).shape
    p = seeds.pos.astype(np.int64)
    z, y, x = p // (Y * X), (p // X) % Y, p % X
    axis = seeds.axis.astype(np.int64)
    own = seeds.label.astype(np.int64)
    coords = {0: (z, y, x), 1: (y, z, x), 2: (x, z, y)}
    for a in (0, 1, 2):
        sa, ra, ca = coords[a]
        for s in np.unique(sa[axis == a]):
            sel = (axis == a) & (sa == s)
            keep[sel] = _adaptive_keep(_slice_view(large_labs[a], a, int(s)), ra[sel], ca[sel], own[sel])
    return keep


def large_labels(work_labels, idx):
    """The cropped label volume as the large walker sees it: the taken
    z-slices with -1 outside their box (for seeds and their variance)."""
    lab = np.array(work_labels, dtype=np.int32, copy=True)
    if not idx:
        return lab, None
    stack = lab[idx]
    y0, y1, x0, x1 = large_slice_box(stack)
    stack[:, :y0] = -1
    stack[:, y1:] = -1
    stack[:, :, :x0] = -1
    stack[:, :, x1:] = -1
    lab[idx] = stack
    return lab, (y0, y1, x0, x1)


def adaptive_seed_mask(large_lab, seeds):
    """pycuda_large.py:513-533 (adaptive random walks): a z-slice seed walks
    iff (row + column) % 4 == 0 or its in-slice window [-100, 100]^2, clipped
    to the interior rows/columns 1..n-2, holds a label that is neither its own
    nor -1. Rows/columns are crop coordinates; large_lab from large_labels."""
    return adaptive_seed_mask_allx({0: large_lab}, seeds)


def subset_seeds(seeds, mask):
    return Seeds(**{f: getattr(seeds, f)[mask] for f in
                    ("pos", "slot", "axis", "label", "b", "var", "rng_cuda", "rng_ocl")})


def _slice_view(vol, axis, s):
    """2-D slice (rows, cols) of a working volume for a seed axis, in the
    row/column convention of the swapped arrays of interpolation.py:212-220."""
    if axis == 0:
        return vol[s]
    if axis == 1:
        return vol[:, s, :]
    return vol[:, :, s]


def extract_seeds(work_img, work_labels, slice_list, all_labels, var_mode="inplane"):
    """Seeds of the listed (axis, slice) entries, ordered by (entry, row, col).

    work_labels: the cropped padded label volume after pre-processing.
    var_mode 'inplane': 3x3 in-slice window (pycuda_small.py:114-131,
    pycuda_small_allx.py:86-105); 'opencl': the extended window of
    pyopencl_small.py:140-185 (adds out-of-plane voxels while fewer than 9).
    """
    Z, Y, X = work_img.shape
    flat = Y * X
    lut = {int(v): i for i, v in enumerate(all_labels)}
    is_float = work_img.dtype == np.float32
    imgf = work_img.astype(F32)
    cols = {k: [] for k in ("pos", "slot", "axis", "label", "b", "var", "rng_cuda", "rng_ocl")}
    stack_count = {0: 0, 1: 0, 2: 0}
    for axis, s in slice_list:
        lab2 = _slice_view(work_labels[axis] if isinstance(work_labels, dict) else work_labels, axis, s)
        img2 = _slice_view(imgf, axis, s)
        R, C = lab2.shape
        stack_idx = stack_count[axis]
        stack_count[axis] += 1
        for r in range(R):
            for c in range(C):
                if axis == 0:
                    z, y, x = s, r, c
                elif axis == 1:
                    z, y, x = r, s, c
                else:
                    z, y, x = r, c, s
                if not (0 < z < Z - 1 and 0 < y < Y - 1 and 0 < x < X - 1):
                    continue
                v = int(lab2[r, c])
                if v < 0 or v not in lut:
                    continue
                B = img2[r, c]
                dev = F32(0.0)
                summe = F32(0.0)
                for n in (-1, 0, 1):
                    for o in (-1, 0, 1):
                        if int(lab2[r + n, c + o]) == v:
                            tmp = F32(B - img2[r + n, c + o])
                            dev = F32(dev + F32(tmp * tmp))
                            summe = F32(summe + F32(1.0))
                if var_mode == "opencl":
                    # pyopencl_small.py:156-178 (z +-1 with x offsets, then z +-1 with y offsets)
                    for n in (-1, 1):
                        for o in (-1, 0, 1):
                            zz, yy, xx = z + n, y, x + o
                            if summe < 9 and int(work_labels[zz, yy, xx]) == v:
                                tmp = F32(B - imgf[zz, yy, xx])
                                dev = F32(dev + F32(tmp * tmp))
                                summe = F32(summe + F32(1.0))
                    for n in (-1, 1):
                        for o in (-1, 1):
                            zz, yy, xx = z + n, y + o, x
                            if summe < 9 and int(work_labels[zz, yy, xx]) == v:
                                tmp = F32(B - imgf[zz, yy, xx])
                                dev = F32(dev + F32(tmp * tmp))
                                summe = F32(summe + F32(1.0))
                var = F32(dev / summe)
                if var < F32(1.0):
                    var = F32(1.0)
                cols["pos"].append(z * flat + y * X + x)
                cols["slot"].append(lut[v])
                cols["axis"].append(axis)
                cols["label"].append(v)
                cols["b"].append(B)
                cols["var"].append(var)
                cols["rng_cuda"].append(stack_idx * R * C + r * C + c)
                cols["rng_ocl"].append(z * flat + y * X + x)
    return Seeds(
        pos=np.asarray(cols["pos"], U32), slot=np.asarray(cols["slot"], U32), axis=np.asarray(cols["axis"], U32),
        label=np.asarray(cols["label"], U32), b=np.asarray(cols["b"], F32), var=np.asarray(cols["var"], F32),
        rng_cuda=np.asarray(cols["rng_cuda"], U32), rng_ocl=np.asarray(cols["rng_ocl"], U32))


# ---------------------------------------------------------------------------
# Walk — NumPy transcription (small cases) and the C oracle
# ---------------------------------------------------------------------------


def walk_numpy(work_img, seeds: Seeds, nbrw, sorw, key, nol):
    """Vectorised over all (seed, walk) pairs; Philox + exp2 weights."""
    Z, Y, X = work_img.shape
    flat = Y * X
    V = Z * flat
    hits = np.zeros(nol * V, np.uint32)
    ns = len(seeds)
    if ns == 0 or nbrw == 0 or sorw == 0:
        return hits.reshape(nol, Z, Y, X)
    img = work_img.reshape(-1)
    is_float = work_img.dtype == np.float32
    sidx = np.tile(np.arange(ns), nbrw)
    walk = np.repeat(np.arange(nbrw, dtype=np.int64), ns)
    pos0 = seeds.pos[sidx].astype(np.int64)
    pos = pos0.copy()
    z = pos // flat
    y = (pos - z * flat) // X
    x = pos - z * flat - y * X
    c = seeds.c[sidx]
    b = seeds.b[sidx]
    base = seeds.slot[sidx].astype(np.int64) * V
    axis, label = seeds.axis[sidx], seeds.label[sidx]
    k0, k1 = int(key) & 0xFFFFFFFF, int(key) >> 32
    offs = np.array([flat, -flat, X, -X, 1, -1], np.int64)
    for st in range(sorw):
        t = walk * sorw + st
        words = philox4x32_10(t >> 2, seeds.pos[sidx], axis, label, k0, k1)
        sub = t & 3
        bits = np.choose(sub, words)
        ws = []
        for off in offs:
            nb = img[pos + off]
            if is_float:
                d = (b - nb.astype(F32)).astype(F32)
                d2 = (d * d).astype(F32)
            else:
                di = b.astype(np.int64) - nb.astype(np.int64)
                d2 = (di * di).astype(F32)
            ws.append(edge_weight(d2, c))
        W0 = ws[0]
        W1 = (W0 + ws[1]).astype(F32)
        W2 = (W1 + ws[2]).astype(F32)
        W3 = (W2 + ws[3]).astype(F32)
        W4 = (W3 + ws[4]).astype(F32)
        W5 = (W4 + ws[5]).astype(F32)
        rnd = (W5 * u01(bits)).astype(F32)
        dirn = np.select(
            [(rnd < W0) | (rnd == 0), (rnd >= W0) & (rnd < W1), (rnd >= W1) & (rnd < W2), (rnd >= W2) & (rnd < W3),
             (rnd >= W3) & (rnd < W4), (rnd >= W4) & (rnd <= W5)], [0, 1, 2, 3, 4, 5], default=-1)
        assert (dirn >= 0).all()
        dz = np.where(dirn == 0, 1, np.where(dirn == 1, -1, 0))
        dy = np.where(dirn == 2, 1, np.where(dirn == 3, -1, 0))
        dx = np.where(dirn == 4, 1, np.where(dirn == 5, -1, 0))
        nz_, ny_, nx_ = z + dz, y + dy, x + dx
        ok = (nz_ > 0) & (nz_ < Z - 1) & (ny_ > 0) & (ny_ < Y - 1) & (nx_ > 0) & (nx_ < X - 1)
        z = np.where(ok, nz_, z)
        y = np.where(ok, ny_, y)
        x = np.where(ok, nx_, x)
        pos = np.where(ok, pos + offs[np.maximum(dirn, 0)], pos)
        np.add.at(hits, (base + pos)[ok], 1)
    return hits.reshape(nol, Z, Y, X)


class _OrSeed(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_uint32), ("slot", ctypes.c_uint32), ("axis", ctypes.c_uint32),
                ("label", ctypes.c_uint32), ("b", ctypes.c_float), ("var", ctypes.c_float),
                ("rng_index", ctypes.c_uint32), ("pad", ctypes.c_uint32)]


_or_dtype = np.dtype([("pos", U32), ("slot", U32), ("axis", U32), ("label", U32), ("b", F32), ("var", F32),
                      ("rng_index", U32), ("pad", U32)])


def build_c_oracle(force=False):
    """Compiles walk_oracle.c (gcc, OpenMP, no FP contraction)."""
    src = HERE / "walk_oracle.c"
    if not force and _LIB.exists() and _LIB.stat().st_mtime >= src.stat().st_mtime:
        return _LIB
    _BUILD.mkdir(exist_ok=True)
    tmp = _LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fsigned-char", "-fPIC", "-shared",
           str(src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB)
    return _LIB


_c = None


def c_oracle():
    global _c
    if _c is None:
        lib = ctypes.CDLL(str(build_c_oracle()))
        lib.or_walk.restype = ctypes.c_int
        lib.or_walk.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        lib.or_weight_exp2.restype = ctypes.c_float
        lib.or_weight_exp2.argtypes = [ctypes.c_float, ctypes.c_float]
        lib.or_weight_constant.restype = ctypes.c_float
        lib.or_weight_constant.argtypes = [ctypes.c_float]
        lib.or_philox.restype = None
        lib.or_philox.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int64]
        _c = lib
    return _c


def walk_c(work_img, seeds: Seeds, nbrw, sorw, key, nol, rng="philox", weight="exp2", rng_index=None,
           nthreads=0):
    """C oracle walk. rng: 'philox' | 'ref_mrg'; weight: 'exp2' | 'ref_expf'.
    rng_index: per-seed MRG init values for rng='ref_mrg'."""
    lib = c_oracle()
    img = np.ascontiguousarray(work_img)
    Z, Y, X = img.shape
    recs = np.zeros(len(seeds), _or_dtype)
    recs["pos"], recs["slot"], recs["axis"], recs["label"] = seeds.pos, seeds.slot, seeds.axis, seeds.label
    recs["b"], recs["var"] = seeds.b, seeds.var
    if rng_index is not None:
        recs["rng_index"] = rng_index
    hits = np.zeros((nol, Z, Y, X), np.uint32)
    rc = lib.or_walk(img.ctypes.data, int(img.dtype == np.float32), Z, Y, X, recs.ctypes.data, len(seeds), nbrw,
                     sorw, int(key), 0 if rng == "philox" else 1, 0 if weight == "exp2" else 1, hits.ctypes.data,
                     nol, nthreads)
    if rc != 0:
        raise ValueError("or_walk rejected its arguments")
    return hits


# ---------------------------------------------------------------------------
# Post-processing (rw_small.py, gpu_kernels.py)
# ---------------------------------------------------------------------------


def smooth_step(phi, update="f32"):
    """One curvature step (gpu_kernels.py:118-183), binary32, reference
    expression order. update 'f32': phi + RN(0.01f * curv); 'ref_f64': the
    reference's `phi += 0.01 * curv` evaluated in binary64 and rounded."""
    phi = np.asarray(phi, F32)
    out = phi.copy()
    p = phi
    c = p[1:-1, 1:-1, 1:-1]
    xm, xp = p[1:-1, 1:-1, :-2], p[1:-1, 1:-1, 2:]
    ym, yp = p[1:-1, :-2, 1:-1], p[1:-1, 2:, 1:-1]
    zm, zp = p[:-2, 1:-1, 1:-1], p[2:, 1:-1, 1:-1]
    c2 = F32(2.0) * c
    dx = (xm - xp) * F32(0.5)
    dxx = (xm - c2) + xp
    dx2 = dx * dx
    dy = (ym - yp) * F32(0.5)
    dyy = (ym - c2) + yp
    dy2 = dy * dy
    dz = (zm - zp) * F32(0.5)
    dzz = (zm - c2) + zp
    dz2 = dz * dz
    dxy = (((p[1:-1, :-2, :-2] + p[1:-1, 2:, 2:]) - p[1:-1, :-2, 2:]) - p[1:-1, 2:, :-2]) * F32(0.25)
    dxz = (((p[2:, 1:-1, :-2] + p[:-2, 1:-1, 2:]) - p[2:, 1:-1, 2:]) - p[:-2, 1:-1, :-2]) * F32(0.25)
    dyz = (((p[2:, :-2, 1:-1] + p[:-2, 2:, 1:-1]) - p[2:, 2:, 1:-1]) - p[:-2, :-2, 1:-1]) * F32(0.25)
    num = dxx * (dy2 + dz2) + dyy * (dx2 + dz2)
    num = num + dzz * (dx2 + dy2)
    num = num - ((F32(2.0) * dx) * dy) * dxy
    num = num - ((F32(2.0) * dx) * dz) * dxz
    num = num - ((F32(2.0) * dy) * dz) * dyz
    den = ((dx2 + dy2) + dz2) + F32(1e-10)
    curv = (num / den).astype(F32)
    if update == "f32":
        out[1:-1, 1:-1, 1:-1] = c + F32(0.01) * curv
    else:
        out[1:-1, 1:-1, 1:-1] = (c.astype(np.float64) + 0.01 * curv.astype(np.float64)).astype(F32)
    return out


def smooth(maps, iters, update="f32"):
    out = np.empty(maps.shape, F32)
    for l in range(maps.shape[0]):
        phi = maps[l].astype(F32)
        for _ in range(iters):
            phi = smooth_step(phi, update)
        out[l] = phi
    return out


def uncertainty(maps):
    """gpu_kernels.py:54-116 + rw_small.py:152-176 on the crop: top-3 in
    label order, uq on the interior (border 0), uint8(uq * 255)."""
    m = maps.astype(F32)
    m0 = np.zeros(m.shape[1:], F32)
    m1 = np.zeros_like(m0)
    m2 = np.zeros_like(m0)
    for l in range(m.shape[0]):
        t = m[l]
        g2 = t > m2
        g1 = ~g2 & (t > m1)
        g0 = ~g2 & ~g1 & (t > m0)
        m0 = np.where(g2, m1, np.where(g1, m1, np.where(g0, t, m0)))
        m1 = np.where(g2, m2, np.where(g1, t, m1))
        m2 = np.where(g2, t, m2)
    mx = np.where(m2 == 0, F32(1.0), m2).astype(F32)
    t0 = (m0 / mx).astype(F32)
    t1 = (m1 / mx).astype(F32)
    a = (F32(1.0) - (F32(1.0) - t0) * (F32(1.0) - t1)).astype(F32)
    uq = np.zeros(m.shape[1:], F32)
    uq[1:-1, 1:-1, 1:-1] = a[1:-1, 1:-1, 1:-1]
    return (uq * F32(255.0)).astype(np.uint8)


# ---------------------------------------------------------------------------
# Whole path, as the reference's small path runs it (interpolation.py:43-284,
# rw_small.py:39-281), with the oracle walk.
# ---------------------------------------------------------------------------


def smart_interpolation(data, labelData, nbrw=10, sorw=4000, smooth_iters=0, allaxis=False, uncertainty_map=False,
                        return_hits=False, denoise=False, only="all", ignore="none", key=0, walker="c",
                        smooth_update="f32", mode="philox", seeding="plain"):
    """The reference's small path with the oracle walk.

    mode 'philox': the product's semantics (Philox stream, exp2 weights,
    binary32 smoothing update). mode 'refstream': the product's
    rng='reference' semantics (the reference's binary32 MRG stream seeded per
    seed as the CUDA walker does, the product's exp2 weights, the smoothing
    update as given). mode 'reference': the reference's own
    randomness and arithmetic (binary32 MRG stream seeded per seed as the CUDA
    walker does, expf weights, binary64 smoothing update) — used to pin this
    restatement against the reference's outputs. seeding 'large': the
    reference large path's seed set (slice skipping, in-plane label box,
    adaptive seeds; biomedisa_helper.py:1068-1080, pycuda_large.py:39-58 and
    :513-533) with the same walk; with allaxis the all-axis large path's
    (every slice with a positive label on each axis, a box per axis,
    adaptive seeds in slice coordinates; biomedisa_helper.py:1082-1099,
    rw_large.py:68-107, pycuda_large_allx.py:37-57 and :513-533)."""
    if mode == "reference":
        smooth_update = "ref_f64"
    labelData, allLabels = pre_processing(labelData, only, ignore)
    data = normalize_image(data)
    if labelData.dtype in (np.uint32, np.int64, np.uint64):
        labelData = labelData.astype(np.int32)
    if denoise:
        data = smooth_img_3x3(data)
    data = np.pad(data, 1)
    labelData = np.pad(labelData, 1)
    zsh, ysh, xsh = data.shape
    if allaxis and slices_adjacent(allaxis_indices(labelData)):
        raise ValueError("At least one empty slice between labels required.")
    az, bz, ay, by, ax, bx = predict_blocksize(labelData)
    data = np.ascontiguousarray(data[az:bz, ay:by, ax:bx])
    lab = np.ascontiguousarray(labelData[az:bz, ay:by, ax:bx])
    if allaxis and seeding == "large":
        slice_list = large_allx_slice_list(lab)
    elif allaxis:
        sl = [(k, 0) for (k, _) in read_indices_allx(lab, 0)]
        t1 = np.ascontiguousarray(np.swapaxes(lab, 0, 1))
        sl += [(k, 1) for (k, _) in read_indices_allx(t1, 1)]
        t2 = np.ascontiguousarray(np.swapaxes(t1, 0, 2))
        sl += [(k, 2) for (k, _) in read_indices_allx(t2, 2)]
        slice_list = [(a, k) for (k, a) in sl]
    elif seeding == "large":
        slice_list = [(0, k) for k in read_labeled_slices_large(lab)]
    else:
        slice_list = [(0, k) for k in read_labeled_slices(lab)[0]]
    if seeding == "large" and allaxis:
        llabs, _ = large_allx_labels(lab, slice_list)
        seeds = extract_seeds(data, llabs, slice_list, allLabels)
        seeds = subset_seeds(seeds, adaptive_seed_mask_allx(llabs, seeds))
    elif seeding == "large":
        llab, _ = large_labels(lab, [k for _, k in slice_list])
        seeds = extract_seeds(data, llab, slice_list, allLabels)
        seeds = subset_seeds(seeds, adaptive_seed_mask(llab, seeds))
    else:
        seeds = extract_seeds(data, lab, slice_list, allLabels)
    nol = len(allLabels)
    if mode == "reference":
        hits = walk_c(data, seeds, nbrw, sorw, key, nol, rng="ref_mrg", weight="ref_expf",
                      rng_index=seeds.rng_cuda)
    elif mode == "refstream":
        hits = walk_c(data, seeds, nbrw, sorw, key, nol, rng="ref_mrg", weight="exp2", rng_index=seeds.rng_cuda)
    elif walker == "numpy":
        hits = walk_numpy(data, seeds, nbrw, sorw, key, nol)
    else:
        hits = walk_c(data, seeds, nbrw, sorw, key, nol)
    res = {"seeds": seeds, "crop": (az, bz, ay, by, ax, bx), "allLabels": allLabels, "slice_list": slice_list,
           "hits_crop": hits}

    def uncrop(vol):
        full = np.zeros((zsh, ysh, xsh), vol.dtype)
        full[az:bz, ay:by, ax:bx] = vol
        return full[1:-1, 1:-1, 1:-1]

    if smooth_iters:
        sm = smooth(hits, smooth_iters, smooth_update)
        if seeding == "large":
            sm[0] = np.maximum(sm[0], 0)  # pycuda_large.py:440-444 clamps label 0's smoothed map at 0
        res["smooth"] = uncrop(get_labels(np.argmax(sm, axis=0).astype(np.uint8), allLabels))
    if uncertainty_map:
        res["uncertainty"] = uncrop(uncertainty(hits))
    if return_hits:
        full = np.zeros((nol, zsh, ysh, xsh), np.float32)
        full[:, az:bz, ay:by, ax:bx] = hits
        res["hits"] = full[:, 1:-1, 1:-1, 1:-1]
    res["regular"] = uncrop(get_labels(np.argmax(hits, axis=0).astype(np.uint8), allLabels))
    return res
