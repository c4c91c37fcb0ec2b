"""Generates tests/golden/ref_cc.npz: label volumes and the outputs of the
reference's own clean() and fill() (biomedisa/features/remove_outlier.py),
imported from the reference tree with stubbed third-party modules. Run in a
container that has the reference checked out (see oracle/ref_import.py).

Usage: python tests/golden/make_golden_cc.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT))


def cases():
    from biomedisa_gb300 import synthetic as S

    rng = np.random.default_rng(11)
    out = {}
    # interpolation-like results: phases with speckle outliers and holes
    for i, (shape, nph) in enumerate((((24, 28, 30), 3), ((32, 20, 26), 5))):
        truth = np.zeros(shape, np.uint8)
        S._phases(rng, truth, nph, size_frac=(0.15, 0.35))
        noise = rng.random(shape)
        t = truth.copy()
        t[noise < 0.02] = rng.integers(0, nph + 1, size=int((noise < 0.02).sum()))
        out[f"phases{i}"] = t
    # nested shells: a label inside another's hole, a hole bigger than the label
    z, y, x = np.mgrid[:30, :30, :30]
    r = np.sqrt((z - 15) ** 2 + (y - 15) ** 2 + (x - 15) ** 2)
    v = np.zeros((30, 30, 30), np.uint8)
    v[(r >= 9) & (r < 11)] = 1
    v[r < 4] = 2
    v[(r >= 12) & (r < 12.8)] = 3
    out["nested"] = v
    # label touching the volume border (box clamped), no label 0 at all
    v = np.full((16, 18, 20), 4, np.uint8)
    v[2:10, 3:12, 0:9] = 7
    v[4:6, 5:8, 2:5] = 4
    v[12:, 15:, 17:] = 9
    out["noback"] = v
    # ties: two components of equal size, a hole as large as the label
    v = np.zeros((12, 12, 12), np.uint8)
    v[1:4, 1:4, 1:4] = 5
    v[7:10, 7:10, 7:10] = 5
    v[1:6, 6:11, 1:6] = 6
    v[2:5, 7:10, 2:5] = 0
    out["ties"] = v
    # random speckle
    out["speckle"] = rng.integers(0, 4, size=(14, 15, 16)).astype(np.uint8)
    return out


def main():
    import ref_import

    data = {}
    with ref_import.reference_modules():
        import importlib

        ro = importlib.import_module("biomedisa.features.remove_outlier")
        for name, vol in cases().items():
            data[f"{name}_in"] = vol
            for thr in (0.1, 0.5):
                data[f"{name}_clean_{thr}"] = ro.clean(vol, thr)
            for thr in (0.9, 0.3):
                try:
                    data[f"{name}_fill_{thr}"] = ro.fill(vol, thr)
                except ValueError:
                    pass  # a label vanished under filling: the reference raises
    np.savez_compressed(ROOT / "tests" / "golden" / "ref_cc.npz", **data)
    print(sorted(data))


if __name__ == "__main__":
    main()
