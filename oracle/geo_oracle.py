"""Geodesic raster-scan interpolation — CPU oracle, TEST INFRASTRUCTURE ONLY.

Only ``tests/`` and the CPU-baseline leg of ``bench.py`` use this module; the
product (``biomedisa_gb300.geodesic``) never does. It restates
``biomedisa/geodis.py``: the scan itself in ``geo_oracle.c`` (literal loops,
numba's scalar typing, see the header there) and ``geodesic_segment``
(:79-104) in NumPy below.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_BUILD = HERE / "_build"
_LIB = _BUILD / "libsi_geo_oracle.so"


def build_geo_oracle(force: bool = False) -> Path:
    """Compiles geo_oracle.c (gcc, no FP contraction)."""
    src = HERE / "geo_oracle.c"
    if not force and _LIB.exists() and _LIB.stat().st_mtime >= src.stat().st_mtime:
        return _LIB
    _BUILD.mkdir(exist_ok=True)
    tmp = _LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", str(src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB)
    return _LIB


_c = None


def _lib():
    global _c
    if _c is None:
        lib = ctypes.CDLL(str(build_geo_oracle()))
        lib.or_geo_scan.restype = ctypes.c_int
        lib.or_geo_scan.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_int]
        _c = lib
    return _c


def raster_scan(img, c, lamb=1.0, iterations=4):
    """geodesic_raster_scan (geodis.py:44-76): updates the float32 array c in
    place from the float32 image img and returns it."""
    if img.dtype != np.float32 or c.dtype != np.float32 or img.shape != c.shape or img.ndim != 3:
        raise TypeError("raster_scan: img and c must be float32 arrays of one 3-D shape")
    if not (img.flags.c_contiguous and c.flags.c_contiguous):
        raise ValueError("raster_scan: arrays must be C-contiguous")
    Z, Y, X = c.shape
    _lib().or_geo_scan(img.ctypes.data, c.ctypes.data, Z, Y, X, float(lamb), int(iterations))
    return c


def geodesic_segment(image, labels):
    """geodesic_segment (geodis.py:79-104). Its lamb and iterations arguments
    are not used by the reference (the scan is called with 1.0 and 4, :97), so
    this restatement takes none."""
    image = image.astype(np.float32)
    image -= np.amin(image)
    image /= np.amax(image)
    all_labels = np.unique(labels)  # biomedisa_helper.unique: the sorted distinct values (:82-103)
    all_labels = all_labels[all_labels >= 0]
    result = np.zeros(labels.shape, np.uint8)
    mask = np.empty(labels.shape, np.float32)
    min_distance = None
    for k, label in enumerate(all_labels):
        mask.fill(np.inf)
        mask[labels == label] = 0
        distance = raster_scan(image, mask, 1.0, 4)
        if k == 0:
            min_distance = distance.copy()
        else:
            tmp = distance < min_distance
            result[tmp] = label
            min_distance[tmp] = distance[tmp]
    return result
