"""Geodesic raster-scan interpolation on one GB300, a drop-in for
``biomedisa.geodis`` (``geodesic_segment``, ``geodesic_raster_scan``,
biomedisa/geodis.py:44-104).

Every label's geodesic distance map is computed at once on the device
(``si_geo_masks`` -> ``si_geo_scan`` -> ``si_geo_select``, declared in
include/smartinterp.h); results are identical to the reference's sequential
numba scan. There is no CPU fallback: without a CUDA device these functions
raise.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .interpolation import _IMG_DTYPES, _LAB_DTYPES, _ptr, _stream, upload


def plan_geo_labels(hist: np.ndarray):
    """The label list of geodesic_segment (geodis.py:89-91: the distinct label
    values without the negative ones, ascending) from the device histogram
    hist[0..255] (values 0..255), hist[256] (negatives), hist[257] (> 255).
    Returns (all_labels uint8, slot_lut int16[256])."""
    if hist[257] > 0:
        raise ValueError("geodesic_segment: label values above 255 are not supported (the result is uint8)")
    all_labels = np.asarray([v for v in range(256) if hist[v] > 0], np.uint8)
    slot_lut = np.full(256, -1, np.int16)
    slot_lut[all_labels] = np.arange(len(all_labels), dtype=np.int16)
    return all_labels, slot_lut


def _labels_for_device(labels: np.ndarray) -> np.ndarray:
    """Integer (or boolean) labels in a dtype the device reads (uint8, int16,
    int32), with every value preserved."""
    ld = np.dtype(labels.dtype)
    if ld in _LAB_DTYPES:
        return np.ascontiguousarray(labels)
    if ld == np.dtype(bool):
        return np.ascontiguousarray(labels, np.uint8)
    if not np.issubdtype(ld, np.integer):
        raise TypeError(f"geodesic_segment: integer labels expected, got {ld}")
    if ld in (np.dtype(np.int8),):
        return np.ascontiguousarray(labels, np.int16)
    if ld == np.dtype(np.uint16):
        return np.ascontiguousarray(labels, np.int32)
    lo, hi = (int(labels.min()), int(labels.max())) if labels.size else (0, 0)
    if lo < -(2 ** 31) or hi > 2 ** 31 - 1:
        raise ValueError("geodesic_segment: label values outside the int32 range")
    return np.ascontiguousarray(labels, np.int32)


def _device(device):
    if not torch.cuda.is_available():
        raise RuntimeError("geodesic interpolation needs a CUDA device; there is no CPU fallback")
    return torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())


SCAN_AUTO, SCAN_WAVEFRONTS, SCAN_CLUSTER, SCAN_WAVEFRONT_GRAPH, SCAN_TILES, SCAN_TILE_GRAPH = range(6)


def scan_device(c: torch.Tensor, img: torch.Tensor, lamb: float = 1.0, iterations: int = 4,
                mode: int = SCAN_AUTO) -> torch.Tensor:
    """geodesic_raster_scan on device tensors: c float32 (nol, Z, Y, X) or
    (Z, Y, X), updated in place; img float32 (Z, Y, X). mode: SCAN_TILES (one
    launch per wavefront of 32x32x8 tiles in skewed coordinates, each tile in
    shared memory), SCAN_TILE_GRAPH (those launches replayed from a cached
    CUDA graph), SCAN_AUTO (SCAN_TILES on the first call with a set of
    arguments, the graph from the second on), SCAN_WAVEFRONTS (one launch per
    voxel wavefront), SCAN_WAVEFRONT_GRAPH, SCAN_CLUSTER (one launch, a
    thread-block cluster per map); all give identical results."""
    if c.dtype != torch.float32 or img.dtype != torch.float32 or not (c.is_cuda and img.is_cuda):
        raise TypeError("scan_device: float32 CUDA tensors expected")
    if img.dim() != 3 or tuple(c.shape[-3:]) != tuple(img.shape) or c.dim() not in (3, 4):
        raise ValueError("scan_device: c must be (Z, Y, X) or (nol, Z, Y, X) over img's shape")
    if not (c.is_contiguous() and img.is_contiguous()) or c.device != img.device:
        raise ValueError("scan_device: contiguous tensors on one device expected")
    Z, Y, X = img.shape
    nol = 1 if c.dim() == 3 else c.shape[0]
    if nol:
        nat.call("si_geo_scan", _ptr(c), _ptr(img), Z, Y, X, nol, float(lamb), int(iterations), int(mode),
                 _stream())
    return c


def scan_launches(shape, lamb: float = 1.0, iterations: int = 4, mode: int = SCAN_AUTO) -> int:
    """Kernel launches one scan of this shape makes (1 in cluster mode), with
    the automatic mode resolved on the current device."""
    import ctypes

    n = ctypes.c_longlong(0)
    nat.call("si_geo_scan_launches", *map(int, shape), float(lamb), int(iterations), int(mode), ctypes.byref(n))
    return int(n.value)


def geodesic_raster_scan(img, c, lamb=1.0, iterations=4):
    """Same call as the reference (geodis.py:44-76): updates the float32
    array ``c`` in place from the float32 image ``img`` and returns it."""
    img = np.asarray(img)
    if not isinstance(c, np.ndarray) or c.dtype != np.float32 or img.dtype != np.float32:
        raise TypeError("geodesic_raster_scan: img and c must be float32 numpy arrays")
    if img.ndim != 3 or img.shape != c.shape:
        raise ValueError("geodesic_raster_scan: img and c must be 3-D arrays of one shape")
    dev = _device(None)
    d_img = torch.from_numpy(np.ascontiguousarray(img)).to(dev)
    d_c = torch.from_numpy(np.ascontiguousarray(c)).to(dev)
    scan_device(d_c, d_img, lamb, iterations)
    c[...] = d_c.cpu().numpy()
    return c


def geodesic_segment_device(img: torch.Tensor, img_dtype: int, lab: torch.Tensor, lab_dtype: int) -> torch.Tensor:
    """geodesic_segment on device-resident (Z, Y, X) tensors of the given
    si_dtype codes; returns the uint8 label volume on the device."""
    if img.dim() != 3 or tuple(lab.shape) != tuple(img.shape):
        raise ValueError("geodesic_segment_device: image and labels must be 3-D volumes of one shape")
    if not (img.is_cuda and lab.is_cuda) or img.device != lab.device or not (img.is_contiguous() and
                                                                              lab.is_contiguous()):
        raise ValueError("geodesic_segment_device: contiguous tensors on one CUDA device expected")
    Z, Y, X = img.shape
    n = Z * Y * X
    dev = img.device
    st = _stream()
    work = torch.empty((Z, Y, X), dtype=torch.float32, device=dev)
    mm = torch.empty(4, dtype=torch.int32, device=dev)
    nat.call("si_geo_normalize", _ptr(img), img_dtype, n, _ptr(work), _ptr(mm), st)
    hist = torch.zeros(258, dtype=torch.int64, device=dev)
    nat.call("si_label_histogram", _ptr(lab), lab_dtype, n, _ptr(hist), st)
    all_labels, slot_lut = plan_geo_labels(hist.cpu().numpy())
    out = torch.zeros((Z, Y, X), dtype=torch.uint8, device=dev)
    nol = len(all_labels)
    if nol == 0:
        return out
    d_lut = torch.from_numpy(slot_lut).to(dev)
    d_lab = torch.from_numpy(all_labels).to(dev)
    c = torch.empty((nol, Z, Y, X), dtype=torch.float32, device=dev)
    nat.call("si_geo_masks", _ptr(lab), lab_dtype, n, _ptr(d_lut), nol, _ptr(c), st)
    # the reference passes lamb=1.0 and iterations=4 whatever its caller asked (geodis.py:97)
    scan_device(c, work, 1.0, 4)
    nat.call("si_geo_select", _ptr(c), nol, n, _ptr(d_lab), _ptr(out), st)
    return out


def geodesic_segment(image, labels, lamb=1.0, iterations=4, *, device=None, return_device=False):
    """Same call as the reference (geodis.py:79-104): the uint8 volume of the
    label whose geodesic (intensity-gradient) distance is smallest, the first
    label of the ascending list mapping to 0. As in the reference, ``lamb``
    and ``iterations`` are not used: the scan always runs with lamb = 1.0 and
    4 iterations. Label values must lie in -2^31..255 (negative values are
    ignored regions); image dtypes other than uint8, int8, uint16, int16,
    int32 and float32 are converted to float32 on the host first, the
    reference's own first step."""
    del lamb, iterations
    image = np.asarray(image)
    labels = np.asarray(labels)
    if image.ndim != 3 or image.shape != labels.shape:
        raise ValueError("geodesic_segment: image and labels must be 3-D arrays of one shape")
    if image.size == 0:
        raise ValueError("geodesic_segment: empty image")
    dev = _device(device)
    if np.dtype(image.dtype) not in _IMG_DTYPES:
        image = image.astype(np.float32)
    image = np.ascontiguousarray(image)
    labels = _labels_for_device(labels)
    img, lab = upload(image, labels, dev)
    out = geodesic_segment_device(img, _IMG_DTYPES[np.dtype(image.dtype)], lab,
                                  _LAB_DTYPES[np.dtype(labels.dtype)])
    if return_device:
        return out
    return out.cpu().numpy()
