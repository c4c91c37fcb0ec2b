"""ctypes binding of libsmartinterp.so (declared in include/smartinterp.h).

The library is required: importing this module without it raises, so no code
path can silently fall back to the CPU.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libsmartinterp.so"

SI_U8, SI_I8, SI_U16, SI_I16, SI_I32, SI_F32 = range(6)

_c_void_p = ctypes.c_void_p
_c_int = ctypes.c_int
_c_u64 = ctypes.c_uint64
_c_u32 = ctypes.c_uint32
_c_float = ctypes.c_float

# name -> argtypes (all return int status unless noted)
_SIGNATURES = {
    "si_label_histogram": [_c_void_p, _c_int, _c_u64, _c_void_p, _c_void_p],
    "si_slice_flags": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_int, _c_void_p, _c_void_p, _c_void_p,
                       _c_void_p, _c_void_p],
    "si_image_minmax": [_c_void_p, _c_int, _c_u64, _c_void_p, _c_void_p],
    "si_prepare_image": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int,
                         _c_float, _c_float, _c_int, _c_void_p, _c_void_p],
    "si_extract_seeds": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int,
                         _c_void_p, _c_void_p, _c_void_p, _c_int, _c_void_p, _c_int, _c_void_p, _c_void_p, _c_void_p,
                         _c_void_p],
    "si_extract_seeds_noalloc": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int,
                                 _c_int, _c_void_p, _c_void_p, _c_void_p, _c_int, _c_void_p, _c_int, _c_void_p,
                                 _c_void_p, _c_void_p],
    "si_extract_seeds_box": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int,
                             _c_int, _c_void_p, _c_void_p, _c_void_p, _c_int, _c_void_p, _c_int, _c_int, _c_int,
                             _c_int, _c_int, _c_void_p, _c_void_p, _c_void_p, _c_void_p],
    "si_adaptive_scratch_bytes": [_c_int, _c_int, _c_int, _c_int, _c_void_p],
    "si_adaptive_seed_filter": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int,
                                _c_int, _c_void_p, _c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int,
                                _c_void_p, _c_void_p, _c_u32, _c_void_p, _c_void_p, _c_void_p, _c_u64, _c_void_p],
    "si_pack_neighbours": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_void_p],
    "si_walk": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_void_p, _c_u32, _c_int, _c_int, _c_u64,
                _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p],
    "si_walk_refstream": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_void_p, _c_u32, _c_int, _c_int,
                          _c_void_p, _c_void_p, _c_int, _c_void_p],
    "si_walk_sorted_set_range": [_c_u64],
    "si_walk_sorted_set_pairs": [_c_int],
    "si_walk_sorted_set_loop": [_c_int],
    "si_walk_sorted_set_round_limit": [_c_u64],
    "si_nn_umma_status": [_c_void_p, _c_void_p],
    "si_nn_conv16_tc_set_streams": [_c_int],
    "si_nn_conv16_tc": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int,
                        _c_int, _c_int, _c_void_p],
    "si_walk_bricks_scratch": [_c_int, _c_int, _c_int, _c_u64, _c_int, _c_void_p],
    "si_walk_bricks": [_c_void_p, _c_int, _c_int, _c_int, _c_void_p, _c_void_p, _c_u32, _c_int, _c_int, _c_u64,
                       _c_void_p, _c_int, _c_void_p, _c_u64, _c_void_p, _c_void_p],
    "si_walk_sorted_scratch": [_c_int, _c_int, _c_int, _c_u64, _c_int, _c_int, _c_void_p],
    "si_walk_sorted": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_void_p, _c_u32, _c_int, _c_int,
                       _c_u64, _c_void_p, _c_int, _c_int, _c_int, _c_void_p, _c_u64, _c_void_p, _c_void_p],
    "si_walk_sorted_batch_scratch": [_c_void_p, _c_int, _c_int, _c_int, _c_void_p],
    "si_walk_sorted_batch": [_c_void_p, _c_int, _c_int, _c_int, _c_u64, _c_int, _c_int, _c_void_p, _c_u64, _c_void_p,
                             _c_void_p],
    "si_argmax": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int,
                  _c_void_p, _c_void_p, _c_void_p, _c_void_p],
    "si_remap_labels": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_void_p,
                        _c_void_p, _c_int, _c_void_p],
    "si_probe_l2_read": [_c_void_p, _c_u64, _c_int, _c_void_p, _c_void_p],
    "si_probe_l2_atomics": [_c_void_p, _c_u64, _c_u64, _c_void_p],
    "si_nn_conv3d_fwd": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int,
                         _c_int, _c_int, _c_int, _c_int, _c_int, _c_void_p],
    "si_nn_wgrad_partial_bytes": [_c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_void_p],
    "si_nn_conv3d_wgrad": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int,
                           _c_int, _c_int, _c_void_p, _c_u64, _c_void_p],
    "si_nn_flip_weights": [_c_void_p, _c_void_p, _c_int, _c_int, _c_void_p],
    "si_nn_relu_bwd": [_c_void_p, _c_void_p, _c_void_p, ctypes.c_int64, _c_void_p],
    "si_nn_xent": [_c_void_p, _c_void_p, _c_void_p, ctypes.c_int64, _c_int, _c_int, _c_float, _c_void_p, _c_void_p,
                   _c_void_p],
    "si_nn_adamw": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, ctypes.c_int64, _c_float, _c_float,
                    _c_float, _c_float, _c_float, _c_int, _c_void_p],
    "si_nn_features": [_c_void_p, _c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int,
                       _c_int, _c_int, _c_void_p, _c_void_p],
    "si_nn_probs": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_int, _c_int, _c_void_p],
    "si_cc_scratch_bytes": [_c_int, _c_int, _c_int, _c_void_p],
    "si_clean": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, ctypes.c_double, _c_int, _c_void_p, _c_u64,
                 _c_void_p],
    "si_fill": [_c_void_p, _c_int, _c_int, _c_int, ctypes.c_double, _c_void_p, _c_int, _c_void_p, _c_u64, _c_void_p],
    "si_smooth_f32": [_c_void_p, _c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_void_p],
    "si_smooth": [_c_void_p, _c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_void_p],
    "si_smooth_tmp_floats": [_c_int, _c_int, _c_int, _c_void_p],
    "si_smooth_status": [_c_void_p, _c_void_p],
    "si_smooth_set_pairs": [_c_int],
    "si_set_wait_limit": [ctypes.c_longlong],
    "si_geo_normalize": [_c_void_p, _c_int, _c_u64, _c_void_p, _c_void_p, _c_void_p],
    "si_geo_masks": [_c_void_p, _c_int, _c_u64, _c_void_p, _c_int, _c_void_p, _c_void_p],
    "si_geo_scan": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, ctypes.c_double, _c_int, _c_int,
                    _c_void_p],
    "si_geo_tile_visit_order": [_c_int, _c_int, _c_int, _c_int, _c_void_p, _c_void_p, _c_void_p],
    "si_geo_scan_launches": [_c_int, _c_int, _c_int, ctypes.c_double, _c_int, _c_int, _c_void_p],
    "si_geo_select": [_c_void_p, _c_int, _c_u64, _c_void_p, _c_void_p, _c_void_p],
    "si_geo_visit_order": [_c_int, _c_int, _c_int, _c_int, _c_void_p],
    "si_extract_seeds_boxes": [_c_void_p, _c_int, *[_c_int] * 9, _c_void_p, _c_void_p, _c_void_p, _c_int, _c_void_p,
                               _c_int, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p],
    "si_adaptive_scratch_bytes_allx": [_c_int, _c_int, _c_int, _c_int, _c_void_p],
    "si_adaptive_seed_filter_allx": [_c_void_p, _c_int, *[_c_int] * 9, _c_void_p, _c_void_p, _c_void_p, _c_int,
                                     _c_void_p, _c_void_p, _c_void_p, _c_u32, _c_void_p, _c_void_p, _c_void_p, _c_u64,
                                     _c_void_p],
    "si_acwe_minmax": [_c_void_p, _c_int, *[_c_int] * 9, _c_void_p, _c_void_p],
    "si_acwe_gather": [_c_void_p, _c_int, *[_c_int] * 7, _c_float, _c_float, _c_void_p, *[_c_int] * 9, _c_void_p,
                       _c_void_p, _c_void_p],
    "si_acwe_label_sums": [_c_void_p, _c_void_p, _c_u64, _c_void_p, _c_void_p],
    "si_acwe_evolution": [_c_void_p, _c_void_p, _c_void_p, ctypes.c_double, _c_int, _c_int, _c_int, _c_void_p,
                          _c_void_p],
    "si_acwe_morph": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_void_p],
    "si_acwe_curvop": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_void_p],
    "si_acwe_scatter": [_c_void_p, *[_c_int] * 9, _c_void_p, _c_void_p],
    "si_acwe_dist_init": [_c_void_p, _c_u64, _c_void_p, _c_void_p],
    "si_acwe_chamfer_band": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_void_p],
    "si_acwe_refine_hist": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_void_p,
                            _c_void_p],
    "si_acwe_refine_decide": [_c_void_p, _c_void_p, _c_int, _c_int, _c_void_p, _c_void_p],
    "si_acwe_refine_apply": [_c_void_p, _c_void_p, _c_void_p, *[_c_int] * 9, _c_void_p, _c_void_p],
}

EXPORTED = ("si_version", "si_last_error", *_SIGNATURES)


class NativeError(RuntimeError):
    """A libsmartinterp entry point returned an error status."""


def load(path: Path | str | None = None) -> ctypes.CDLL:
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build it with `python -m biomedisa_gb300.build` (nvcc, sm_103a). "
            "There is no CPU fallback."
        )
    lib = ctypes.CDLL(str(p))
    lib.si_version.restype = _c_int
    lib.si_version.argtypes = []
    lib.si_last_error.restype = ctypes.c_char_p
    lib.si_last_error.argtypes = []
    for name, args in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = _c_int
        fn.argtypes = args
    return lib


_lib: ctypes.CDLL | None = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        _lib = load()
    return _lib


CALLS: dict[str, int] = {}  # entry-point call counts (measurement bookkeeping)


def call(name: str, *args) -> None:
    """Calls an entry point and raises NativeError on a non-zero status."""
    L = lib()
    CALLS[name] = CALLS.get(name, 0) + 1
    rc = getattr(L, name)(*args)
    if rc != 0:
        msg = L.si_last_error().decode(errors="replace")
        raise NativeError(f"{name} failed ({rc}): {msg}")
