"""Generates tests/golden/ref_acwe.npz: inputs and outputs of the reference's
own active-contour post-processing (biomedisa/features/active_contour.py:
activeContour with simple=False, the 'acwe' result, and simple=True, the
'refined' result; curvop_numba.py: evolution, erosion, dilation, curvop),
imported from the reference tree with stubbed third-party modules. numba is
absent, so the reference's function bodies run as Python with numba's scalar
typing restored where NumPy 2 differs (oracle/ref_import.py: _numba_typed).
Run in a container that has the reference checked out.

Usage: python tests/golden/make_golden_acwe.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT))


def cases():
    """name -> (image, labels, alpha, smooth, steps)."""
    from biomedisa_gb300.synthetic import blob_volume as blobs

    out = {}
    img, lab = blobs((18, 22, 26), 1, [1, 2], [(8, 9, 9), (9, 12, 17)], [(6, 6, 7), (5, 7, 6)], 12.0)
    out["u8"] = (img, lab.astype(np.uint8), 1.0, 1, 3)
    img, lab = blobs((16, 20, 21), 2, [3, 7, 9], [(7, 6, 6), (8, 13, 14), (4, 14, 5)], [(5, 4, 4), (5, 5, 6),
                     (3, 4, 3)], 20.0, dtype=np.float32)
    out["f32_alpha"] = (img, lab.astype(np.uint8), 0.6, 2, 2)
    # a long x axis: activeContour's +-100 crop (reduce_blocksize) cuts x
    img, lab = blobs((8, 10, 236), 3, [5, 200], [(4, 5, 110), (4, 4, 124)], [(3, 4, 9), (3, 3, 6)], 10.0)
    out["crop_x"] = (img, lab.astype(np.uint8), 1.0, 1, 2)
    # every voxel labelled (no label 0): label 0 is added by pre_processing
    img, lab = blobs((10, 12, 14), 4, [2], [(5, 6, 7)], [(4, 4, 5)], 9.0)
    lab[lab == 0] = 1
    out["nozero"] = (img, lab.astype(np.uint8), 1.0, 1, 2)
    # labels touching every face of the volume, alpha > 1
    img, lab = blobs((12, 13, 15), 5, [1, 4], [(0, 6, 7), (11, 12, 0)], [(6, 5, 6), (5, 6, 7)], 15.0)
    out["edges"] = (img, lab.astype(np.uint8), 1.7, 3, 1)
    return out


def main():
    import ref_import

    data = {}
    with ref_import.reference_modules():
        import importlib

        ac = importlib.import_module("biomedisa.features.active_contour")
        for name, (img, lab, alpha, smooth, steps) in cases().items():
            data[f"{name}_image"] = img
            data[f"{name}_labels"] = lab
            data[f"{name}_params"] = np.array([alpha, smooth, steps], np.float64)
            data[f"{name}_acwe"] = ac.activeContour(img.copy(), lab.copy(), alpha, smooth, steps)
            data[f"{name}_refined"] = ac.activeContour(img.copy(), lab.copy(), simple=True)
            changed = int(np.count_nonzero(data[f"{name}_acwe"] != lab))
            print(name, "acwe changed", changed, "refined labels", np.bincount(data[f"{name}_refined"].ravel()))
    np.savez_compressed(ROOT / "tests" / "golden" / "ref_acwe.npz", **data)
    print(sorted(data))


if __name__ == "__main__":
    main()
