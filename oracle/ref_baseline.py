"""Timed CPU baseline: the reference's own CPU path for the walk — its OpenCL
walker ``randomWalk`` (pyopencl_small.py:137-316, the path the reference takes
on a CPU OpenCL device and for all-axis input), compiled as C with OpenMP
(oracle/_ref/libref_fast.so) — on a bounded sample of a workload.
Test/baseline infrastructure only: bench.py's CPU-baseline leg and reference
arm use it; the product never does.

The launch loop restates pyopencl_small._walk_on_current_gpu (:80-135): int8
image (uint8 - 128) or float32, a full-volume uchar label array holding
``ignore_value`` outside the seeded pixels, one launch per label, int32 hits.
The sample keeps the seeds of a band of rows of the first labelled z-slice;
steps = seeds * nbrw * sorw (every seed walks for its own label only).
"""
from __future__ import annotations

import ctypes
import os
import time

import numpy as np

from ref_run import ref_lib

import oracle


def _threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def ocl_walk_sample(work_img, work_labels, all_labels, nbrw, sorw, z_slice, rows):
    """Runs the reference OpenCL walker over the seeds of rows [rows[0], rows[1])
    of crop slice z_slice. Returns (steps, seconds, seeds)."""
    lib = ref_lib("fast")
    Z, Y, X = work_img.shape
    all_labels = [int(v) for v in all_labels]
    ignore_value = next(i for i in range(256) if i not in set(all_labels))
    lab = np.full((Z, Y, X), ignore_value, np.uint8)
    r0, r1 = rows
    band = work_labels[z_slice, r0:r1].astype(np.int64)
    band = np.where(band < 0, ignore_value, band).astype(np.uint8)
    lab[z_slice, r0:r1] = band
    if work_img.dtype == np.uint8:
        raw = (work_img.astype(np.int16) - 128).astype(np.int8)
        variant = 0
    else:
        raw = work_img.astype(np.float32)
        variant = 1
    hits = np.zeros((Z, Y, X), np.int32)
    planes = np.asarray([z_slice], np.int32)
    interior = np.zeros((Y, X), bool)
    interior[1:-1, 1:-1] = True
    seeds = 0
    if 0 < z_slice < Z - 1:
        seg = work_labels[z_slice]
        seeds = int(np.count_nonzero(interior[r0:r1] & np.isin(seg[r0:r1], all_labels)))
    dt = 0.0
    for seg in all_labels:
        hits.fill(0)  # the per-label enqueue_fill_buffer; not part of the timed walk
        t0 = time.perf_counter()
        lib.ref_ocl_walk_planes(variant, planes.ctypes.data_as(ctypes.c_void_p), 1, Z, Y, X, seg,
                                raw.ctypes.data_as(ctypes.c_void_p), lab.ctypes.data_as(ctypes.c_void_p),
                                hits.ctypes.data_as(ctypes.c_void_p), X, Y, Z, sorw, nbrw)
        dt += time.perf_counter() - t0
    return seeds * nbrw * sorw, dt, seeds


def bounded_sample(work_img, work_labels, all_labels, z_slice, nbrw, sorw, target_seconds=12.0):
    """Calibrates on a few rows, then times a band sized for ~target_seconds.
    Returns a dict with steps/s, cores and the sample description."""
    Y = work_img.shape[1]
    mid = Y // 2
    rows = 4
    steps, dt, seeds = ocl_walk_sample(work_img, work_labels, all_labels, nbrw, sorw, z_slice, (mid, mid + rows))
    rate = steps / max(dt, 1e-6)
    per_row = max(steps / rows, 1.0)
    want = int(min(max(target_seconds * rate / per_row, 1), Y - 2))
    r0 = max(1, mid - want // 2)
    r1 = min(Y - 1, r0 + want)
    steps, dt, seeds = ocl_walk_sample(work_img, work_labels, all_labels, nbrw, sorw, z_slice, (r0, r1))
    return {
        "value": steps / dt,
        "unit": "walker-steps/s",
        "cores": _threads(),
        "seconds": dt,
        "steps": steps,
        "kind": "reference",
        "sample": f"reference OpenCL walker (C, OpenMP) on the {seeds} seeds of rows {r0}-{r1} of crop z-slice "
                  f"{z_slice}, all {len(all_labels)} labels, nbrw={nbrw}, sorw={sorw}",
    }


def port_walk_sample(work_img, work_labels, all_labels, nbrw, sorw, z_slice, rows, nthreads=0):
    """The oracle's C walker switched to the reference OpenCL kernel's
    semantics (its RNG seeded by the global voxel index, expf weights, the
    extended variance window; pinned bit for bit to the reference kernel by
    tests/test_oracle_pin.py) over the seeds of rows [rows[0], rows[1]) of crop
    slice z_slice. Returns (steps, seconds, seeds)."""
    r0, r1 = rows
    lab = np.full(work_labels.shape, -1, work_labels.dtype)
    zs = slice(max(z_slice - 1, 0), z_slice + 2)
    ys = slice(max(r0 - 1, 0), r1 + 1)
    lab[zs, ys] = work_labels[zs, ys]
    seeds = oracle.extract_seeds(work_img, lab, [(0, z_slice)], all_labels, var_mode="opencl")
    Y, X = work_img.shape[1:]
    row = (seeds.pos.astype(np.int64) // X) % Y
    keep = (row >= r0) & (row < r1)
    seeds = oracle.Seeds(**{k: getattr(seeds, k)[keep] for k in
                            ("pos", "slot", "axis", "label", "b", "var", "rng_cuda", "rng_ocl")})
    t0 = time.perf_counter()
    oracle.walk_c(work_img, seeds, nbrw, sorw, 0, len(all_labels), rng="ref_mrg", weight="ref_expf",
                  rng_index=seeds.rng_ocl, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return len(seeds) * nbrw * sorw, dt, len(seeds)


def bounded_sample_port(work_img, work_labels, all_labels, z_slice, nbrw, sorw, target_seconds=12.0):
    """bounded_sample with the oracle's restatement of the reference kernel,
    for hosts where oracle/_ref cannot be built (no reference tree and no
    extracted sources)."""
    Y = work_img.shape[1]
    mid = Y // 2
    rows = 4
    cores = _threads()
    steps, dt, seeds = port_walk_sample(work_img, work_labels, all_labels, nbrw, sorw, z_slice, (mid, mid + rows),
                                        cores)
    rate = steps / max(dt, 1e-6)
    per_row = max(steps / rows, 1.0)
    want = int(min(max(target_seconds * rate / per_row, 1), Y - 2))
    r0 = max(1, mid - want // 2)
    r1 = min(Y - 1, r0 + want)
    steps, dt, seeds = port_walk_sample(work_img, work_labels, all_labels, nbrw, sorw, z_slice, (r0, r1), cores)
    return {
        "value": steps / dt,
        "unit": "walker-steps/s",
        "cores": cores,
        "seconds": dt,
        "steps": steps,
        "kind": "port",
        "sample": f"the oracle's C restatement of the reference OpenCL walker (OpenMP) on the {seeds} seeds of rows "
                  f"{r0}-{r1} of crop z-slice {z_slice}, all {len(all_labels)} labels, nbrw={nbrw}, sorw={sorw}",
    }
