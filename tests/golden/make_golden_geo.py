"""Generates tests/golden/ref_geo.npz: inputs and outputs of the reference's
own geodesic interpolation (biomedisa/geodis.py: geodesic_segment and
geodesic_raster_scan), imported from the reference tree with stubbed
third-party modules. numba is absent, so the reference's function bodies run
as Python on float32 views that follow numba's scalar typing
(oracle/ref_import.py: _NumbaF32). Run in a container that has the reference
checked out.

Usage: python tests/golden/make_golden_geo.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT))


def segment_cases():
    """name -> (image, labels) for geodesic_segment."""
    from biomedisa_gb300 import synthetic as S

    out = {}
    img, lab, _ = S.plain_volume(seed=3, shape=(10, 12, 14), z_every=3, semi=(2, 5))
    out["u8"] = (img, lab)
    rng = np.random.default_rng(5)
    # uint16, labels with gaps, an ignored (negative) region, no label on most slices
    img = rng.integers(0, 60000, size=(9, 11, 13)).astype(np.uint16)
    img[:, :, 6:] += 3000
    lab = np.zeros(img.shape, np.int32)
    lab[0, 2:9, 2:6] = 3
    lab[0, 2:9, 7:11] = 7
    lab[8, 3:7, 3:10] = 7
    lab[4, 1:4, 1:4] = -1
    out["u16_gaps"] = (img, lab)
    # float32 of arbitrary range; no label 0 (the first label found maps to 0)
    img = (rng.normal(size=(8, 10, 9)) * 40.0 - 7.0).astype(np.float32)
    lab = np.zeros(img.shape, np.int16)
    lab[1, 2:8, 1:8] = 2
    lab[6, 1:5, 2:7] = 5
    lab[lab == 0] = 2
    lab[3:5, :, :] = 9
    out["f32_nozero"] = (img, lab)
    # constant image: the normalisation divides 0 by 0 (NaN everywhere)
    img = np.full((6, 7, 8), 17, np.uint8)
    lab = np.zeros(img.shape, np.int32)
    lab[2, 2:5, 2:6] = 1
    out["const"] = (img, lab)
    # thin volumes: two z-slices; one z-slice (no pass runs)
    img = rng.integers(0, 255, size=(2, 5, 6)).astype(np.uint8)
    lab = np.zeros(img.shape, np.int32)
    lab[0, 1:3, 1:4] = 4
    out["thin2"] = (img, lab)
    img = rng.integers(0, 255, size=(1, 5, 6)).astype(np.uint8)
    out["thin1"] = (img, np.where(lab[:1] > 0, 4, 0).astype(np.int32))
    return out


def scan_cases():
    """name -> (img, c, lamb, iterations) for geodesic_raster_scan."""
    rng = np.random.default_rng(9)
    out = {}
    img = rng.random((7, 9, 8)).astype(np.float32)
    c = np.full(img.shape, np.inf, np.float32)
    c[0, 3, 4] = 0.0
    c[6, 1:3, 1:5] = 0.0
    out["lamb1_it4"] = (img, c, 1.0, 4)
    c = np.full(img.shape, np.inf, np.float32)
    c[3, 4, 3] = 0.0
    out["lamb05_it2"] = (img, c.copy(), 0.5, 2)
    out["lamb0_it1"] = (img, c.copy(), 0.0, 1)
    c = rng.random(img.shape).astype(np.float32) * 3.0
    out["lamb07_random_c"] = (img, c, 0.7, 3)
    return out


def main():
    import ref_import

    data = {}
    with ref_import.reference_modules():
        import importlib

        geo = importlib.import_module("biomedisa.geodis")
        for name, (img, lab) in segment_cases().items():
            data[f"seg_{name}_image"] = img
            data[f"seg_{name}_labels"] = lab
            data[f"seg_{name}_result"] = geo.geodesic_segment(img.copy(), lab.copy())
            print("segment", name, np.bincount(data[f"seg_{name}_result"].ravel()))
        for name, (img, c, lamb, it) in scan_cases().items():
            data[f"scan_{name}_img"] = img
            data[f"scan_{name}_c"] = c
            data[f"scan_{name}_params"] = np.array([lamb, it], np.float64)
            data[f"scan_{name}_out"] = geo.geodesic_raster_scan(img.copy(), c.copy(), lamb, it)
            print("scan", name, np.isfinite(data[f"scan_{name}_out"]).sum())
    np.savez_compressed(ROOT / "tests" / "golden" / "ref_geo.npz", **data)
    print(sorted(data))


if __name__ == "__main__":
    main()
