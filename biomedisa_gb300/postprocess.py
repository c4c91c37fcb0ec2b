"""Outlier removal and hole filling of label volumes on the device
(si_clean / si_fill), the reference's biomedisa/features/remove_outlier.py
clean (:67-105) and fill (:107-141), and the result keys that
rw_small.py:223-243 derives from them."""
from __future__ import annotations

import ctypes

import torch

from . import _native as nat


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _scratch(shape, device):
    need = ctypes.c_uint64(0)
    nat.call("si_cc_scratch_bytes", *shape, ctypes.byref(need))
    return torch.empty(int(need.value), dtype=torch.uint8, device=device), int(need.value)


def present_labels(labels: torch.Tensor) -> list[int]:
    """Ascending label values present in a uint8 volume (the reference's unique())."""
    counts = torch.bincount(labels.reshape(-1).to(torch.int64), minlength=256)
    return [int(v) for v in torch.nonzero(counts).flatten().tolist()]


def clean(labels: torch.Tensor, threshold: float = 0.1) -> torch.Tensor:
    """remove_outlier.clean on a uint8 device volume; returns a new volume."""
    if labels.dtype != torch.uint8 or labels.dim() != 3 or not labels.is_cuda:
        raise ValueError("clean takes a 3-D uint8 label volume on a CUDA device")
    labels = labels.contiguous()
    present = present_labels(labels)
    skip = present[0] if present else -1
    out = torch.empty_like(labels)
    scratch, nbytes = _scratch(tuple(labels.shape), labels.device)
    nat.call("si_clean", labels.data_ptr(), out.data_ptr(), *labels.shape, float(threshold), skip,
             scratch.data_ptr(), nbytes, _stream())
    return out


def fill(labels: torch.Tensor, threshold: float = 0.9) -> torch.Tensor:
    """remove_outlier.fill on a uint8 device volume; returns a new volume."""
    if labels.dtype != torch.uint8 or labels.dim() != 3 or not labels.is_cuda:
        raise ValueError("fill takes a 3-D uint8 label volume on a CUDA device")
    out = labels.contiguous().clone()
    todo = present_labels(out)[1:]
    if not todo:
        return out
    lst = (ctypes.c_int * len(todo))(*todo)
    scratch, nbytes = _scratch(tuple(out.shape), out.device)
    nat.call("si_fill", out.data_ptr(), *out.shape, float(threshold), lst, len(todo), scratch.data_ptr(), nbytes,
             _stream())
    return out


def post_results(res: dict, clean_threshold=None, fill_threshold=None) -> dict:
    """Adds 'cleaned', 'smooth_cleaned', 'filled' and 'cleaned_filled' to a
    result dict of device tensors as rw_small.py:223-243 does (a threshold
    that is None or 0 disables its step, like the reference's truth test)."""
    regular = res["regular"]
    if clean_threshold:
        res["cleaned"] = clean(regular, clean_threshold)
        if "smooth" in res:
            res["smooth_cleaned"] = clean(res["smooth"], clean_threshold)
    if fill_threshold:
        res["filled"] = fill(regular, fill_threshold)
    if clean_threshold and fill_threshold:
        res["cleaned_filled"] = res["cleaned"] + (res["filled"] - regular)  # uint8 wrap-around, as numpy
    return res
