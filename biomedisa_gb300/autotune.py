"""Autotuner for the sorted-sweep walker's tile and queue parameters.

The walker's results do not depend on these parameters (integer hit sums), only
its speed does: the sort-brick edge (walkers are bucketed by label and brick of
edge^3 voxels between sweeps) and the sweep length (steps per sweep launch).
The tuner times every candidate on the caller's own volumes with shortened
walks (4 sweeps of every walk), keeps the fastest, and caches the choice per
workload signature in a JSON file ($SI_AUTOTUNE_CACHE or
~/.cache/biomedisa_gb300/autotune.json).
"""
from __future__ import annotations

import ctypes
import json
import math
import os
import tempfile
import threading
from pathlib import Path

import torch

from . import _native as nat

CANDIDATES = ((6, 32), (8, 32), (4, 32), (6, 24), (6, 48), (10, 32))


def cache_path() -> Path:
    p = os.environ.get("SI_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "biomedisa_gb300" / "autotune.json"


def signature(vols, nbrw: int, sorw: int, walks: int) -> str:
    """Workload class: device, record kind, walk counts and sizes (log2 bins)."""
    dev = torch.cuda.get_device_name()
    kinds = sorted({int(v.work_is_float) for v in vols})
    vox = sum(v.Zc * v.Yc * v.Xc for v in vols)
    return json.dumps([dev, kinds, len(vols), nbrw, sorw, int(math.log2(max(walks, 1))),
                       int(math.log2(max(vox, 1)))])


def _load() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


_STORE_LOCK = threading.Lock()


def _store(key: str, value) -> None:
    """Adds one entry; the file is replaced atomically, so a concurrent reader
    sees the old or the new cache, never a partial one. Threads of one process
    take turns (the read-modify-write keeps every thread's entry), and each
    write goes through its own uniquely named temporary file."""
    with _STORE_LOCK:
        data = _load()
        data[key] = value
        path = cache_path()
        tmp = None
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            with tempfile.NamedTemporaryFile("w", dir=path.parent, prefix=path.name + ".", suffix=".tmp",
                                             delete=False) as f:
                tmp = f.name
                f.write(json.dumps(data, indent=1))
            os.replace(tmp, path)
            tmp = None
        except OSError:
            pass
        finally:
            if tmp is not None:
                try:
                    os.unlink(tmp)
                except OSError:
                    pass


def tune(vol_array, n_vols: int, hits: list, nbrw: int, sorw: int, key: int, walks: int, use_cache: bool = True):
    """Returns (sort_edge, sweep_steps, report). hits are zeroed afterwards."""
    vols = [vol_array[i] for i in range(n_vols)]
    sig = signature(vols, nbrw, sorw, walks)
    if use_cache:
        hit = _load().get(sig)
        if hit:
            return int(hit["sort_edge"]), int(hit["sweep_steps"]), {"cached": True, **hit}
    stream = torch.cuda.current_stream()
    results = []
    for edge, steps in CANDIDATES:
        probe = min(sorw, 4 * steps)
        need = ctypes.c_ulonglong(0)
        nat.call("si_walk_sorted_batch_scratch", vol_array, n_vols, nbrw, edge, ctypes.byref(need))
        scratch = torch.empty(max(int(need.value), 1), dtype=torch.uint8, device="cuda")
        for h in hits:
            h.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        rounds = ctypes.c_int(0)
        s.record(stream)
        nat.call("si_walk_sorted_batch", vol_array, n_vols, nbrw, probe, key, steps, edge, scratch.data_ptr(),
                 int(need.value), ctypes.byref(rounds), stream.cuda_stream)
        e.record(stream)
        torch.cuda.synchronize()
        rate = walks * probe / (s.elapsed_time(e) / 1e3)
        results.append({"sort_edge": edge, "sweep_steps": steps, "steps_per_s": rate})
        del scratch
    for h in hits:
        h.zero_()
    best = max(results, key=lambda r: r["steps_per_s"])
    _store(sig, best)
    return best["sort_edge"], best["sweep_steps"], {"cached": False, "candidates": results, **best}
