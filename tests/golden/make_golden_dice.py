"""Generates tests/golden/ref_dice.npz: the REFERENCE's own labels, with its own
walker kernels and its own random stream, on benchmark configurations.

The reference's smart_interpolation (Python host code unmodified, its CUDA
kernel sources compiled for the CPU by oracle/ref_extract.py, pycuda and
mpi4py faked by oracle/ref_run.py) is run on
  * ``plain128``: the plain single-volume configuration in full — uint8 128^3,
    background mean 60 plus two ellipsoids (means 130 and 200, semi-axes
    U[15, 45]), N(0, 15) noise, labels 0..2 on every 10th z-slice,
    nbrw=10, sorw=4000, smooth=0 (``synthetic.plain_volume(seed=0)``);
  * ``plain128_allaxis``: the same volume labelled on all three axes (every 10th
    z-slice, every 16th y- and x-slice), allaxis=True, nbrw=10, sorw=4000,
    smooth=20;
  * ``slab``: a reduced slab of the all-axis configuration — uint8
    (z, y, x) = (96, 128, 128) from the same generator (8 phases, N(0, 12)
    noise, 3-voxel blur at the interfaces), labels on every 8th XY and every
    16th YZ / XZ slice, allaxis=True, nbrw=10, sorw=4000, smooth=100
    (``synthetic.allaxis_volume(seed=0, shape=(96, 128, 128))``).
Only the outputs and SHA-256 digests of the inputs are stored; the test
regenerates the inputs with the same seeded generator and checks the digests.
The reference's walk draws from a different random stream than this
package's Philox stream, so the test compares label volumes by per-label
Dice, not bit for bit.

Cases already in the file are kept; --force recomputes every case.

Usage: python tests/golden/make_golden_dice.py [--force]   (about 12 minutes on 8 cores)
"""
from __future__ import annotations

import contextlib
import hashlib
import io
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import ref_run  # noqa: E402

from biomedisa_gb300.synthetic import allaxis_volume, plain_volume, sparse_labels  # noqa: E402

PLAIN_128 = dict(nbrw=10, sorw=4000, smooth=0, allaxis=False)
PLAIN_128_ALLAXIS = dict(nbrw=10, sorw=4000, smooth=20, allaxis=True)
SLAB_SHAPE = (96, 128, 128)
SLAB = dict(nbrw=10, sorw=4000, smooth=100, allaxis=True)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def cases():
    img, lab, truth = plain_volume(seed=0)
    yield "plain128", img, lab, PLAIN_128
    yield "plain128_allaxis", img, sparse_labels(truth.astype(np.int32), z_every=10, y_every=16, x_every=16), PLAIN_128_ALLAXIS
    img, lab, _ = allaxis_volume(seed=0, shape=SLAB_SHAPE)
    yield "slab", img, lab, SLAB


def main() -> None:
    path = HERE / "ref_dice.npz"
    out = {} if "--force" in sys.argv or not path.exists() else dict(np.load(path))
    for name, img, lab, kw in cases():
        if f"{name}_regular" in out and str(out[f"{name}_img_sha256"]) == digest(img) and \
                str(out[f"{name}_lab_sha256"]) == digest(lab):
            continue
        t = time.time()
        with contextlib.redirect_stdout(io.StringIO()):
            res = ref_run.reference_smart_interpolation(img, lab, **kw)
        print(f"{name}: reference run {time.time() - t:.1f} s", flush=True)
        out[f"{name}_img_sha256"] = np.array(digest(img))
        out[f"{name}_lab_sha256"] = np.array(digest(lab))
        out[f"{name}_regular"] = res["regular"]
        if "smooth" in res:
            out[f"{name}_smooth"] = res["smooth"]
        np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
