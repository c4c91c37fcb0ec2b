"""Active-contour post-processing on one GB300: the reference's
``activeContour`` (biomedisa/features/active_contour.py:109-202) in both of
its modes, as run by ``smart_interpolation(acwe=True)`` (rw_small.py:246-255,
rw_large.py:262-271):

  * 'acwe' (simple=False): ``steps`` rounds of label means, one evolution pass
    and, for every label, ``smooth`` erosion/dilation pairs
    (curvop_numba.py:5-149);
  * 'refined' (simple=True): the chamfer band (distance <= 10) around the
    labels, per-slice Gaussian likelihoods of the band's label and non-label
    intensities, and the per-slice relabelling of the band (:204-225).

All work is device kernels of libsmartinterp (si_acwe_*); the
host computes the crop box and the label list from two small device reads.
There is no CPU fallback.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .interpolation import _IMG_DTYPES, _LAB_DTYPES, _err, _ptr, _stream, normalize_host_dtypes, plan_labels, upload

# reduce_blocksize's margin around the labels' bounding box (active_contour.py:86-103)
CROP_MARGIN = 100
# refinement band: distance <= this after the chamfer scan (active_contour.py:209-210)
BAND_DISTANCE = 10.0


def crop_box(bbox, padded_shape):
    """reduce_blocksize (active_contour.py:84-104) from the nonzero labels'
    bounding box (zmin, zmax, ymin, ymax, xmin, xmax) in padded coordinates;
    returns (z0, y0, x0, Zc, Yc, Xc)."""
    lo_hi = []
    for a, s in enumerate(padded_shape):
        lo, hi = int(bbox[2 * a]), int(bbox[2 * a + 1])
        if hi < 0:  # no nonzero label: the reference's untouched initial values
            lo, hi = s, 0
        lo = lo - CROP_MARGIN if lo - CROP_MARGIN > 0 else 0
        hi = hi + CROP_MARGIN if hi + CROP_MARGIN < s else s
        lo_hi.append((lo, hi))
    (z0, z1), (y0, y1), (x0, x1) = lo_hi
    return z0, y0, x0, z1 - z0, y1 - y0, x1 - x0


class Frame:
    """Where an image array sits in the padded frame: its voxel (a, b, c) is
    padded voxel (z0 + a, y0 + b, x0 + c)."""

    def __init__(self, img: torch.Tensor, code: int, origin, dims):
        self.img, self.code = img, code
        self.z0, self.y0, self.x0 = (int(v) for v in origin)
        self.Z, self.Y, self.X = (int(v) for v in dims)

    def covers(self, Z, Y, X) -> bool:
        """True when the array covers the whole interior 1..Z x 1..Y x 1..X."""
        return (self.z0 <= 1 and self.z0 + self.Z - 1 >= Z and self.y0 <= 1 and self.y0 + self.Y - 1 >= Y
                and self.x0 <= 1 and self.x0 + self.X - 1 >= X)


def _u8_conversion(frame: Frame, Z, Y, X):
    """img_to_uint8 (biomedisa_helper.py:345-352) parameters: (convert, mn, mx)
    with mx = amax - amin in binary32; the image as the reference sees it is
    the array, zero outside it."""
    if frame.code == nat.SI_U8:
        return 0, 0.0, 1.0
    mm = torch.tensor([np.inf, -np.inf], dtype=torch.float32, device=frame.img.device)
    nat.call("si_acwe_minmax", _ptr(frame.img), frame.code, frame.Z, frame.Y, frame.X, frame.z0, frame.y0, frame.x0,
             Z, Y, X, _ptr(mm), _stream())
    lo, hi = (np.float32(v) for v in mm.cpu().numpy())
    if not frame.covers(Z, Y, X):
        lo, hi = min(lo, np.float32(0)), max(hi, np.float32(0))
    return 1, float(lo), float(np.float32(hi - lo))


class AcweRun:
    """One active-contour call on device tensors. ``labels``: uint8 (Z, Y, X)
    device tensor; ``all_labels``: the reference's bm.allLabels (sorted, label
    0 first unless removed by ``ignore``)."""

    def __init__(self, frame: Frame, labels: torch.Tensor, all_labels):
        if labels.dtype != torch.uint8 or labels.dim() != 3:
            raise ValueError("labels must be a uint8 3-D device tensor")
        self.dev = labels.device
        self.frame, self.labels = frame, labels.contiguous()
        self.all_labels = [int(v) for v in all_labels]
        self.Z, self.Y, self.X = (int(s) for s in labels.shape)
        self.launches = 0

    def _box(self):
        Z, Y, X = self.Z, self.Y, self.X
        nz = torch.from_numpy((np.arange(256) != 0).astype(np.uint8)).to(self.dev)
        fz = torch.zeros(Z + 2, dtype=torch.uint8, device=self.dev)
        imax = np.iinfo(np.int32).max
        bbox = torch.tensor([imax, -1, imax, -1, imax, -1], dtype=torch.int32, device=self.dev)
        nat.call("si_slice_flags", _ptr(self.labels), nat.SI_U8, Z, Y, X, _ptr(nz), 0, _ptr(fz), None, None,
                 _ptr(bbox), _stream())
        self.launches += 1
        return crop_box(bbox.cpu().numpy(), (Z + 2, Y + 2, X + 2))

    def gather(self):
        """The crop box and the uint8 crops D (image) and L (labels)."""
        Z, Y, X = self.Z, self.Y, self.X
        self.box = self._box()
        convert, mn, mx = _u8_conversion(self.frame, Z, Y, X)
        self.launches += int(convert)
        z0, y0, x0, cZ, cY, cX = self.box
        n = cZ * cY * cX
        self.D = torch.empty(n, dtype=torch.uint8, device=self.dev)
        self.L = torch.empty(n, dtype=torch.uint8, device=self.dev)
        f = self.frame
        nat.call("si_acwe_gather", _ptr(f.img), f.code, f.Z, f.Y, f.X, f.z0, f.y0, f.x0, convert, mn, mx,
                 _ptr(self.labels), Z, Y, X, z0, y0, x0, cZ, cY, cX, _ptr(self.D), _ptr(self.L), _stream())
        self.launches += 1

    def acwe(self, alpha=1.0, smooth=1, steps=3) -> torch.Tensor:
        """active_contour.py:188-197, then the crop put back (:185-188)."""
        z0, y0, x0, cZ, cY, cX = self.box
        n = cZ * cY * cX
        # self.L stays the gathered labels (refined() reads it too)
        L, tmp = self.L.clone(), torch.empty_like(self.L)
        sums = torch.zeros(512, dtype=torch.int64, device=self.dev)
        for _ in range(int(steps)):
            sums.zero_()
            nat.call("si_acwe_label_sums", _ptr(self.D), _ptr(L), n, _ptr(sums), _stream())
            nat.call("si_acwe_evolution", _ptr(L), _ptr(self.D), _ptr(sums), float(alpha), cZ, cY, cX, _ptr(tmp),
                     _stream())
            L, tmp = tmp, L
            self.launches += 2
            for k in self.all_labels:
                nat.call("si_acwe_curvop", _ptr(L), _ptr(tmp), cZ, cY, cX, k, int(smooth), _stream())
                self.launches += 2 * int(smooth)
        out = torch.empty((self.Z, self.Y, self.X), dtype=torch.uint8, device=self.dev)
        nat.call("si_acwe_scatter", _ptr(L), z0, y0, x0, cZ, cY, cX, self.Z, self.Y, self.X, _ptr(out), _stream())
        self.launches += 1
        return out

    def refined(self, scan_events=None) -> torch.Tensor:
        """refinement (active_contour.py:204-225), then the crop put back.
        scan_events: optional pair of CUDA events recorded around the chamfer
        band (for measurement)."""
        z0, y0, x0, cZ, cY, cX = self.box
        n = cZ * cY * cX
        dist = torch.empty(n, dtype=torch.float32, device=self.dev)
        nat.call("si_acwe_dist_init", _ptr(self.L), n, _ptr(dist), _stream())
        # the chamfer band (active_contour.py:45-81 and :209-210) by Jacobi
        # relaxation, exact for every voxel that reaches the result
        spare = torch.empty(n, dtype=torch.float32, device=self.dev)
        if scan_events:
            scan_events[0].record()
        nat.call("si_acwe_chamfer_band", _ptr(dist), _ptr(spare), cZ, cY, cX, _stream())
        if scan_events:
            scan_events[1].record()
        del spare
        cands = self.all_labels[1:]
        class_lut = np.zeros(256, np.int16)
        for j, v in enumerate(cands):
            class_lut[v] = j + 1
        ncls = len(cands) + 1
        hist = torch.zeros(cZ * ncls * 256, dtype=torch.int32, device=self.dev)
        nat.call("si_acwe_refine_hist", _ptr(dist), _ptr(self.D), _ptr(self.L),
                 _ptr(torch.from_numpy(class_lut).to(self.dev)), ncls, cZ, cY, cX, _ptr(hist), _stream())
        lut = torch.empty(cZ * 256, dtype=torch.uint8, device=self.dev)
        cand = torch.from_numpy(np.asarray(cands if cands else [0], np.uint8)).to(self.dev)
        nat.call("si_acwe_refine_decide", _ptr(hist), _ptr(cand), len(cands), cZ, _ptr(lut), _stream())
        out = torch.empty((self.Z, self.Y, self.X), dtype=torch.uint8, device=self.dev)
        nat.call("si_acwe_refine_apply", _ptr(dist), _ptr(self.D), _ptr(lut), z0, y0, x0, cZ, cY, cX, self.Z, self.Y,
                 self.X, _ptr(out), _stream())
        self.launches += 15
        return out


def label_list(labels: torch.Tensor) -> list[int]:
    """bm.allLabels of pre_processing (biomedisa_helper.py:671-694) for a uint8
    label volume: the values present, with 0 first."""
    hist = torch.zeros(258, dtype=torch.int64, device=labels.device)
    nat.call("si_label_histogram", _ptr(labels), nat.SI_U8, labels.numel(), _ptr(hist), _stream())
    h = hist.cpu().numpy()
    vals = [v for v in range(256) if h[v] > 0]
    return vals if vals and vals[0] == 0 else [0] + vals


def acwe_results(frame: Frame, labels: torch.Tensor, alpha=1.0, smooth=1, steps=3):
    """The 'acwe' and 'refined' results of smart_interpolation for a device
    uint8 result volume (rw_small.py:246-252): both activeContour calls on the
    same image and labels. Returns (acwe, refined) device tensors, or
    (None, None) where the reference's pre_processing rejects the labels."""
    all_labels = label_list(labels)
    if len(all_labels) < 2:
        _err("No labeled slices found.")
        return None, None
    run = AcweRun(frame, labels, all_labels)
    run.gather()
    a = run.acwe(alpha, smooth, steps)
    r = run.refined()
    return a, r


def activeContour(data, labelData, alpha=1.0, smooth=1, steps=3, path_to_data=None, path_to_labels=None,
                  compression=True, ignore="none", only="all", simple=False, queue=4, img_id=None, friend_id=None,
                  remote=False, *, device=None, return_device=False):
    """activeContour (active_contour.py:109-202) on one GB300: same arguments
    and result (uint8 labels of the input shape; 'refined' when simple=True,
    else 'acwe'); errors print 'Error: ...' and return None. File I/O,
    Django and queue arguments are accepted and ignored; pass arrays.
    Labels follow pre_processing (biomedisa_helper.py:639-723): float labels
    become int32, values > 255 become 0, ``only`` / ``ignore`` set labels to
    0; negative labels are rejected (the reference keeps them in the volume
    and indexes its mean table with them)."""
    if data is None or labelData is None:
        raise NotImplementedError("loading volumes from files is outside this package; pass numpy arrays")
    if not torch.cuda.is_available():
        raise RuntimeError("activeContour needs a CUDA device; there is no CPU fallback")
    data = np.asarray(data)
    labelData = np.asarray(labelData)
    if labelData.ndim != 3:
        return _err("Label data must be three-dimensional.")
    if data.shape != labelData.shape:
        return _err("Image and label data must have the same x,y,z-dimensions.")
    data, labelData = normalize_host_dtypes(data, labelData)
    img, lab = upload(data, labelData, device)
    lab_code = _LAB_DTYPES[np.dtype(labelData.dtype)]
    hist = torch.zeros(258, dtype=torch.int64, device=lab.device)
    nat.call("si_label_histogram", _ptr(lab), lab_code, lab.numel(), _ptr(hist), _stream())
    h = hist.cpu().numpy()
    if h[256] > 0:
        raise ValueError("negative labels are not supported by activeContour on this path")
    plan = plan_labels(h, only, ignore)
    if plan.nol < 2:
        return _err("No labeled slices found.")
    # value -> label after pre_processing (removed values and values > 255 -> 0)
    keep = np.zeros(258, np.uint8)
    for v in range(256):
        keep[v] = v if (v in set(int(x) for x in plan.all_labels) or v == 0) else 0
    lut = torch.from_numpy(keep).to(lab.device)
    idx = lab.to(torch.int64).clamp_(max=257) if lab_code != nat.SI_U8 else lab.to(torch.int64)
    lab8 = lut[idx].contiguous()
    Z, Y, X = labelData.shape
    frame = Frame(img, _IMG_DTYPES[np.dtype(data.dtype)], (1, 1, 1), (Z, Y, X))
    run = AcweRun(frame, lab8, plan.all_labels)
    run.gather()
    out = run.refined() if simple else run.acwe(alpha, smooth, steps)
    return out if return_device else out.cpu().numpy()
