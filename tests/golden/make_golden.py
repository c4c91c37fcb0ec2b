"""Generates the golden fixtures in tests/golden/ from the REFERENCE itself.

Runs in the development container, where the reference tree is mounted:
the reference's own smart_interpolation (Python host code unmodified, its
CUDA kernel sources compiled for the CPU by oracle/ref_extract.py, pycuda and
mpi4py faked by oracle/ref_run.py) and its own host helpers
(biomedisa_helper.py) are called on small seeded inputs, and inputs plus
outputs are stored as compressed .npz files. The tests read only these files,
so they run anywhere.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import contextlib
import io
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import ref_run  # noqa: E402
from ref_import import reference_modules  # noqa: E402

from biomedisa_gb300.synthetic import plain_volume, sparse_labels  # noqa: E402


def _quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def pipeline_cases():
    """(name, image, labels, kwargs) for the reference pipeline."""
    cases = []
    img, lab, truth = plain_volume(seed=1, shape=(40, 36, 34), z_every=5, semi=(6, 12))
    kw = dict(nbrw=2, sorw=60, smooth=3, uncertainty=True, return_hits=True)
    cases.append(("plain_u8", img, lab, kw))
    cases.append(("plain_u16", img.astype(np.uint16) * 3 + 7, lab, kw))
    cases.append(("plain_i8_denoise", (img.astype(np.int16) - 128).astype(np.int8), lab,
                  dict(kw, denoise=True, smooth=0)))
    cases.append(("plain_f32_denoise", img.astype(np.float32) * 0.37 - 5.0, lab, dict(kw, denoise=True, smooth=2)))
    # four phases, negative (ignored) regions, a value > 255, only/ignore
    rng = np.random.default_rng(5)
    img2, _, truth2 = plain_volume(seed=2, shape=(34, 38, 36), z_every=4, semi=(6, 12))
    t2 = truth2.astype(np.int32)
    t2[(t2 == 0) & (rng.random(t2.shape) < 0.02)] = 3
    t2[5:9, 5:12, 5:12] = 4
    lab2 = sparse_labels(t2, z_every=4)
    lab2[8, 2:6, 2:6] = -1
    lab2[12, 30:33, 30:33] = 300
    cases.append(("labels_neg_big", img2, lab2, dict(kw, smooth=2)))
    cases.append(("labels_only", img2, lab2, dict(kw, only="1,2", smooth=0)))
    cases.append(("labels_ignore", img2, lab2, dict(kw, ignore="3", smooth=0)))
    # all-axis seeds (z every 6th, y and x every 9th)
    img3, _, truth3 = plain_volume(seed=4, shape=(38, 40, 36), z_every=6, semi=(7, 13))
    lab3 = sparse_labels(truth3.astype(np.int32), z_every=6, y_every=9, x_every=9)
    cases.append(("allaxis_u8", img3, lab3, dict(kw, allaxis=True, smooth=2)))
    cases.append(("allaxis_u16", img3.astype(np.uint16) * 5, lab3, dict(kw, allaxis=True, smooth=0)))
    return cases


def make_pipeline():
    for name, img, lab, kw in pipeline_cases():
        res = _quiet(ref_run.reference_smart_interpolation, img, lab, **kw)
        out = {"image": img, "labels": lab}
        for k, v in res.items():
            out["out_" + k] = v
        np.savez_compressed(HERE / f"ref_pipeline_{name}.npz", kwargs=repr(kw), **out)
        print(name, sorted(res))


def make_helpers():
    """Fixtures of the reference's host helpers on random label volumes."""
    rng = np.random.default_rng(11)
    out = {}
    with reference_modules():
        h = ref_run.reference_helpers()
        for i in range(6):
            shape = tuple(int(s) for s in rng.integers(8, 20, 3))
            arr = np.zeros(shape, np.int32)
            # lines, blobs and full slices
            for _ in range(4):
                z = int(rng.integers(0, shape[0]))
                arr[z, rng.integers(0, shape[1]), :] = int(rng.integers(1, 4))
                arr[z, :, rng.integers(0, shape[2])] = int(rng.integers(1, 4))
            z = int(rng.integers(0, shape[0]))
            arr[z] = rng.integers(0, 3, shape[1:])
            y = int(rng.integers(0, shape[1]))
            arr[:, y, :] = rng.integers(0, 3, (shape[0], shape[2]))
            out[f"allx_in_{i}"] = arr
            for ax, a in enumerate((arr, np.ascontiguousarray(np.swapaxes(arr, 0, 1)),
                                    np.ascontiguousarray(np.swapaxes(np.swapaxes(arr, 0, 1), 0, 2)))):
                idx, data = h.read_labeled_slices_allx(a, ax)
                out[f"allx_idx_{i}_{ax}"] = np.asarray([k for k, _ in idx], np.int32)
                out[f"allx_data_{i}_{ax}"] = data
                out[f"allx_ind_{i}_{ax}"] = np.asarray([k for k, _ in h.read_indices_allx(a, ax)], np.int32)
            idx, data = h.read_labeled_slices(arr)
            out[f"rls_idx_{i}"] = np.asarray(idx, np.int32)

            class BM:
                pass

            bm = BM()
            bm.labelData = np.pad(arr, 1)
            bm = h.predict_blocksize(bm)
            out[f"bbox_{i}"] = np.asarray([bm.argmin_z, bm.argmax_z, bm.argmin_y, bm.argmax_y, bm.argmin_x,
                                           bm.argmax_x], np.int64)
        # get_labels incl. the case where index 0 is absent
        pre = rng.integers(1, 4, (5, 6, 7)).astype(np.uint8)
        out["gl_in_noz"] = pre
        out["gl_out_noz"] = h.get_labels(pre, np.asarray([0, 5, 9, 200]))
        pre2 = rng.integers(0, 4, (5, 6, 7)).astype(np.uint8)
        out["gl_in"] = pre2
        out["gl_out"] = h.get_labels(pre2, np.asarray([0, 5, 9, 200]))
        # pre_processing variants
        for j, (only, ignore) in enumerate((("all", "none"), ("2,5", "none"), ("all", "5,7"), ("all", "0"))):
            lab = rng.integers(-2, 9, (6, 7, 8)).astype(np.int32)
            lab[0, 0, 0] = 400
            bm = BM()
            bm.data = np.zeros(lab.shape, np.uint8)
            bm.labelData = lab.copy()
            bm.only, bm.ignore = only, ignore
            bm.django_env = False
            bm.slicer = False
            bm.path_to_data = None
            bm = _quiet(h.pre_processing, bm)
            out[f"pp_in_{j}"] = lab
            out[f"pp_lab_{j}"] = bm.labelData
            out[f"pp_all_{j}"] = np.asarray(bm.allLabels, np.int64)
            out[f"pp_opt_{j}"] = np.asarray([only, ignore])
        # smooth_img_3x3 (numba function run as Python)
        u8 = rng.integers(0, 256, (5, 6, 7)).astype(np.uint8)
        out["den_u8_in"] = u8
        out["den_u8_out"] = h.smooth_img_3x3(u8)
        f32 = rng.uniform(0, 255, (5, 6, 7)).astype(np.float32)
        out["den_f32_in"] = f32
        out["den_f32_out"] = h.smooth_img_3x3(f32)
        gt = rng.integers(0, 3, (6, 6, 6))
        rs = rng.integers(0, 3, (6, 6, 6))
        out["dice_gt"], out["dice_rs"] = gt, rs
        out["dice"] = np.asarray(h.Dice_score(gt, rs))
    np.savez_compressed(HERE / "ref_helpers.npz", **out)
    print("helpers", len(out))


if __name__ == "__main__":
    make_helpers()
    make_pipeline()
