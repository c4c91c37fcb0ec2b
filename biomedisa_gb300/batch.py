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
                            normalize_host_dtypes, upload)


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


def walk_batch(jobs, nbrw, sorw, rng_seed, sort_edge=0, sweep_steps=0, tune=True):
    """One batched walk over all prepared jobs. Returns a report dict."""
    live = [j for j in jobs if j is not None]
    if not live:
        return {}
    arr = (SiVolume * len(live))()
    for k, j in enumerate(live):
        cp = j.cplan
        arr[k] = SiVolume(_ptr(j.packed), _ptr(j.hits), _ptr(j.seeds), _ptr(j.n_seeds), j.seed_capacity, cp.Zc,
                          cp.Yc, cp.Xc, j.lplan.nol, int(j.work_is_float))
    walks = sum(int(j.n_seeds.item()) for j in live) * nbrw
    report = {}
    if tune and not (sort_edge and sweep_steps):
        sort_edge, sweep_steps, report = autotune.tune(arr, len(live), [j.hits for j in live], nbrw, sorw,
                                                        rng_seed, walks)
    need = ctypes.c_ulonglong(0)
    nat.call("si_walk_sorted_batch_scratch", arr, len(live), nbrw, sort_edge, ctypes.byref(need))
    scratch = torch.empty(max(int(need.value), 1), dtype=torch.uint8, device="cuda")
    rounds = ctypes.c_int(0)
    nat.call("si_walk_sorted_batch", arr, len(live), nbrw, sorw, rng_seed, sweep_steps, sort_edge,
             _ptr(scratch), int(need.value), ctypes.byref(rounds), _stream())
    for j in live:
        j.rounds = int(rounds.value)
    report.update({"sort_edge": sort_edge, "sweep_steps": sweep_steps, "sweeps": int(rounds.value),
                   "walker_steps": walks * sorw})
    return report


def smooth_batch(jobs, graph=True):
    """All volumes' smoothing iterations, captured once in a CUDA graph and
    replayed (graph=False launches them directly)."""
    live = [j for j in jobs if j is not None and j.smooth]
    if not live:
        return
    vmax = max(j.cplan.voxels for j in live)
    tmp0 = torch.empty(vmax, dtype=torch.float32, device="cuda")
    tmp1 = torch.empty(vmax, dtype=torch.float32, device="cuda")
    if not graph:
        for j in live:
            j.smooth_launch(tmp0, tmp1)
        return
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        for j in live:
            j.smooth_launch(tmp0, tmp1)
    g.replay()
    torch.cuda.current_stream().synchronize()


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
