"""Batched smart interpolation: many volumes of uneven size in one pass.

All volumes' walks (every label, every seed) advance together in the same
sorted-sweep launches (si_walk_sorted_batch); the smoothing iterations of all
volumes are captured once into a CUDA graph and replayed; the walker's sort
and sweep parameters come from the autotuner. Every volume's result equals
smart_interpolation on that volume alone (same rng_seed).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as nat
from . import autotune
from .interpolation import (DEFAULT_RNG_SEED, DeviceJob, _IMG_DTYPES, _LAB_DTYPES, _err, _ptr, _stream,
                            normalize_host_dtypes, smooth_buffers, smooth_check, smooth_tmp_floats, upload)


class SiVolume(ctypes.Structure):
    """si_volume_t of include/smartinterp.h."""

    _fields_ = [("packed", ctypes.c_void_p), ("hits", ctypes.c_void_p), ("seeds", ctypes.c_void_p),
                ("n_seeds", ctypes.c_void_p), ("max_seeds", ctypes.c_uint32), ("Zc", ctypes.c_int),
                ("Yc", ctypes.c_int), ("Xc", ctypes.c_int), ("nol", ctypes.c_int), ("work_is_float", ctypes.c_int)]


def prepare_jobs(volumes, labels, nbrw, sorw, smooth, allaxis, uncertainty, denoise, only, ignore, rng_seed):
    """Uploads, analyses and prepares every volume; None where the reference
    would report an error (the message is printed)."""
    dev = []
    for img, lab in zip(volumes, labels):
        img, lab = np.asarray(img), np.asarray(lab)
        if lab.ndim != 3:
            _err("Label data must be three-dimensional.")
            dev.append(None)
            continue
        if img.shape != lab.shape:
            _err("Image and label data must have the same x,y,z-dimensions.")
            dev.append(None)
            continue
        data, labd = normalize_host_dtypes(img, lab)
        ti, tl = upload(data, labd)
        dev.append((ti, _IMG_DTYPES[data.dtype], tl, _LAB_DTYPES[labd.dtype]))
    return prepare_device_jobs(dev, nbrw, sorw, smooth, allaxis, uncertainty, denoise, only, ignore, rng_seed)


def prepare_device_jobs(device_volumes, nbrw, sorw, smooth, allaxis, uncertainty, denoise, only, ignore, rng_seed):
    """Like prepare_jobs for volumes already on the device: a list of
    (image tensor, image dtype code, label tensor, label dtype code) or None."""
    jobs = []
    for item in device_volumes:
        if item is None:
            jobs.append(None)
            continue
        ti, icode, tl, lcode = item
        job = DeviceJob(ti, icode, tl, lcode, nbrw=nbrw, sorw=sorw, allaxis=allaxis, smooth=smooth,
                        uncertainty=uncertainty, denoise=denoise, only=only, ignore=ignore, rng_seed=rng_seed,
                        walker="sorted")
        msg = job.analyze()
        if msg:
            _err(msg)
            jobs.append(None)
            continue
        job.prepare()
        cp = job.cplan
        job.hits = torch.zeros((job.lplan.nol, cp.Zc, cp.Yc, cp.Xc), dtype=torch.int32, device=job.dev)
        jobs.append(job)
    return jobs


def run_device_batch(device_volumes, nbrw=10, sorw=4000, smooth=0, allaxis=False, uncertainty=False,
                     return_hits=False, denoise=False, only="all", ignore="none", rng_seed=DEFAULT_RNG_SEED,
                     sort_edge=0, sweep_steps=0, autotune_params=True, graph=True):
    """The whole batch on device-resident volumes; returns (jobs, results of
    device tensors, report)."""
    jobs = prepare_device_jobs(device_volumes, nbrw, sorw, smooth, allaxis, uncertainty, denoise, only, ignore,
                               rng_seed)
    rep = walk_batch(jobs, nbrw, sorw, rng_seed, sort_edge, sweep_steps, tune=autotune_params)
    results = [None if j is None else j.post_regular(return_hits) for j in jobs]
    if smooth:
        smooth_batch(jobs, graph=graph)
        for j, r in zip(jobs, results):
            if j is not None:
                r["smooth"] = j.post_smooth()
    return jobs, results, rep


GROUP_WALKS = 1 << 25  # walks per group of consecutive volumes (compact working set per sweep)


def volume_groups(seeds, nbrw, group_walks=GROUP_WALKS):
    """Consecutive volume index ranges holding about group_walks walks each
    (a volume is never split)."""
    groups, start, acc = [], 0, 0
    for k, n in enumerate(seeds):
        acc += n * nbrw
        if acc >= group_walks:
            groups.append((start, k + 1))
            start, acc = k + 1, 0
    if start < len(seeds):
        groups.append((start, len(seeds)))
    return groups


def walk_batch(jobs, nbrw, sorw, rng_seed, sort_edge=0, sweep_steps=0, tune=True, group_walks=GROUP_WALKS):
    """Batched walk over all prepared jobs: volumes are walked in groups of
    consecutive volumes of about group_walks walks, all labels and volumes of
    a group sharing every launch (si_walk_sorted_batch). Hits are integer sums
    of independent walks, so the grouping does not change them. Returns a
    report dict."""
    live = [j for j in jobs if j is not None]
    if not live:
        return {}
    arr = (SiVolume * len(live))()
    for k, j in enumerate(live):
        cp = j.cplan
        arr[k] = SiVolume(_ptr(j.packed), _ptr(j.hits), _ptr(j.seeds), _ptr(j.n_seeds), j.seed_capacity, cp.Zc,
                          cp.Yc, cp.Xc, j.lplan.nol, int(j.work_is_float))
    seeds = [int(j.n_seeds.item()) for j in live]
    walks = sum(seeds) * nbrw
    report = {}
    if tune and not (sort_edge and sweep_steps):
        sort_edge, sweep_steps, report = autotune.tune(arr, len(live), [j.hits for j in live], nbrw, sorw,
                                                        rng_seed, walks)
    groups = volume_groups(seeds, nbrw, group_walks) if group_walks else [(0, len(live))]
    size = ctypes.sizeof(SiVolume)
    need_max = 0
    for a, b in groups:
        need = ctypes.c_ulonglong(0)
        nat.call("si_walk_sorted_batch_scratch", ctypes.byref(arr, a * size), b - a, nbrw, sort_edge,
                 ctypes.byref(need))
        need_max = max(need_max, int(need.value))
    scratch = torch.empty(max(need_max, 1), dtype=torch.uint8, device="cuda")
    total_rounds = 0
    for a, b in groups:
        rounds = ctypes.c_int(0)
        nat.call("si_walk_sorted_batch", ctypes.byref(arr, a * size), b - a, nbrw, sorw, rng_seed, sweep_steps,
                 sort_edge, _ptr(scratch), need_max, ctypes.byref(rounds), _stream())
        total_rounds += int(rounds.value)
    for j in live:
        j.rounds = total_rounds
    report.update({"sort_edge": sort_edge, "sweep_steps": sweep_steps, "sweeps": total_rounds,
                   "walker_steps": walks * sorw, "volume_groups": len(groups)})
    return report


def smooth_batch(jobs, graph=True):
    """All volumes' smoothing iterations, captured once in a CUDA graph and
    replayed (graph=False launches them directly)."""
    live = [j for j in jobs if j is not None and j.smooth]
    if not live:
        return
    nmax = max(smooth_tmp_floats(j.cplan.Zc, j.cplan.Yc, j.cplan.Xc) for j in live)
    tmp0, tmp1 = smooth_buffers(1, 1, 1, "cuda", floats=nmax)
    if not graph:
        for j in live:
            j.smooth_launch(tmp0, tmp1)
        smooth_check()
        return
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        for j in live:
            j.smooth_launch(tmp0, tmp1)
    g.replay()
    smooth_check()


def smart_interpolation_batch(volumes, labels, nbrw=10, sorw=4000, smooth=0, allaxis=False, uncertainty=False,
                              return_hits=False, denoise=False, only="all", ignore="none",
                              rng_seed=DEFAULT_RNG_SEED, sort_edge=0, sweep_steps=0, autotune_params=True,
                              graph=True, return_device=False, report=None):
    """Smart interpolation of a list of (image, labels) volumes in one batch.

    Returns a list with one result dict per volume (None where the reference
    would report an error), each identical to smart_interpolation on that
    volume with the same rng_seed. ``report`` (a dict) receives the tuner's
    choice and the number of sweeps."""
    if not torch.cuda.is_available():
        raise RuntimeError("smart_interpolation_batch needs a CUDA device; there is no CPU fallback")
    jobs = prepare_jobs(volumes, labels, nbrw, sorw, smooth, allaxis, uncertainty, denoise, only, ignore, rng_seed)
    rep = walk_batch(jobs, nbrw, sorw, rng_seed, sort_edge, sweep_steps, tune=autotune_params)
    results = [None if j is None else j.post_regular(return_hits) for j in jobs]
    if smooth:
        smooth_batch(jobs, graph=graph)
        for j, r in zip(jobs, results):
            if j is not None:
                r["smooth"] = j.post_smooth()
    if report is not None:
        report.update(rep)
    if return_device:
        return results
    return [None if r is None else {k: v.cpu().numpy() for k, v in r.items()} for r in results]
