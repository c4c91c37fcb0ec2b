"""CPU oracle of the reference's outlier removal and hole filling — TEST
INFRASTRUCTURE ONLY (imported by tests/ and the fixture generator, never by
the product).

Restates biomedisa/features/remove_outlier.py:
  * reduce_blocksize (:45-65): bounding box of the non-zero voxels grown by one
    voxel and clamped to the volume;
  * clean (:67-105): per label after the smallest, 6-connected components of
    the label's mask; components larger than threshold x the largest one are
    kept, the others become 0;
  * fill (:107-141): per label after the smallest, in ascending order and on
    the image as modified by the previous labels: 6-connected components of
    the complement of the label inside its grown bounding box (connectivity
    does not leave the box); the largest entry of [label size, component
    sizes...] (first maximum, so the label itself wins ties) is left alone,
    every component larger than threshold x label size is left alone, and
    everything else in the box becomes the label (the label's own voxels
    become 0 if the label itself was the largest entry);
  * the 'cleaned_filled' result of rw_small.py:239-240, cleaned + (filled -
    regular) in uint8 arithmetic.
Connected components use scipy.ndimage.label, the reference's own routine.
One difference: a label that vanished because an earlier label's filling
covered it is skipped here; the reference raises (argmax of an empty array).
"""
from __future__ import annotations

import numpy as np
from scipy import ndimage

STRUCT6 = np.array([[[0, 0, 0], [0, 1, 0], [0, 0, 0]],
                    [[0, 1, 0], [1, 1, 1], [0, 1, 0]],
                    [[0, 0, 0], [0, 1, 0], [0, 0, 0]]])


def labels_present(image):
    """The reference's unique() for non-negative integer volumes (biomedisa_helper.py:82-103)."""
    return np.nonzero(np.bincount(image.ravel().astype(np.int64)))[0]


def grown_bbox(mask):
    """remove_outlier.py:45-65 (the bounds, not the copy)."""
    Z, Y, X = mask.shape
    nz = np.nonzero(mask)
    if nz[0].size == 0:
        return None
    lo = [max(int(a.min()) - 1, 0) for a in nz]
    hi = [min(int(a.max()) + 1, s - 1) + 1 for a, s in zip(nz, (Z, Y, X))]
    return lo, hi


def clean(image, threshold=0.1):
    out = np.array(image, copy=True, order="C")
    for k in labels_present(out)[1:]:
        label = out == k
        lo, hi = grown_bbox(label)
        sl = tuple(slice(a, b) for a, b in zip(lo, hi))
        comp, _ = ndimage.label(label[sl], structure=STRUCT6)
        size = np.bincount(comp.ravel())
        biggest = size[1:].max()
        keep = np.zeros(size.size, bool)
        keep[1:] = size[1:] > threshold * biggest
        region = np.zeros_like(label)
        region[sl] = keep[comp]
        out[label] = 0
        out[region] = k
    return out


def fill(image, threshold=0.9):
    out = np.array(image, copy=True, order="C")
    for k in labels_present(out)[1:]:
        label = out == k
        box = grown_bbox(label)
        if box is None:
            continue  # vanished under an earlier label's filling (the reference raises here)
        lo, hi = box
        sl = tuple(slice(a, b) for a, b in zip(lo, hi))
        reduced = label[sl].astype(np.uint8)
        label_size = int(reduced.sum())
        comp, _ = ndimage.label(1 - reduced, structure=STRUCT6)
        size = np.bincount(comp.ravel())
        biggest = int(np.argmax(size))
        filled = np.ones_like(reduced)
        filled[comp == biggest] = 0
        for l in range(1, size.size):
            if size[l] > threshold * label_size and l != biggest:
                filled[comp == l] = 0
        region = np.zeros_like(label)
        region[sl] = filled == 1
        out[label] = 0
        out[region] = k
    return out


def cleaned_filled(cleaned, filled, regular):
    return (cleaned.astype(np.uint8) + (filled.astype(np.uint8) - regular.astype(np.uint8))).astype(np.uint8)
