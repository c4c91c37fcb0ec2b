"""GB300 smart interpolation: the drop-in for
``biomedisa.interpolation.smart_interpolation`` (biomedisa/interpolation.py:43-284).

Host logic mirrors the reference's small path (pre-processing, dtype
normalisation, one-voxel pad, all-axis checks, +-100 bounding-box crop,
labelled-slice selection, argmax/get_labels, optional smoothing and
uncertainty); every O(volume) step runs as a CUDA kernel of
libsmartinterp.so on one GPU. Differences from the reference, by design:
  * randomness is Philox4x32-10 keyed by (rng_seed, label, seed voxel, step)
    instead of the binary32 MRG recurrence; edge weights use the library's
    own exp2 evaluation; hits are exact uint32 counts;
  * the smoothing update phi + 0.01*kappa is evaluated in binary32 (the
    reference's literal 0.01 is binary64);
  * every volume takes the plain full walk (the reference switches to its
    seed-subsampling large path above 2e9 bytes, interpolation.py:196);
  * file I/O, MPI ranks and Django are not part of this path; clean, fill
    (postprocess.py) and acwe (active_contour.py) run on the device.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as nat

DEFAULT_RNG_SEED = 0x243F6A8885A308D3
WALKERS = ("auto", "sorted", "tiles", "packed")
SEEDINGS = ("plain", "large")
SEED_RECORD_BYTES = 16


def _err(message: str):
    """Reference error behaviour: print 'Error: ...' and return None
    (biomedisa_helper.py:622-637 with bm.success = False)."""
    print("Error:", message)
    return None


# update arithmetic of the smoothing step (include/smartinterp.h si_smooth_update)
SMOOTH_UPDATES = {"f32": 0, "ref_f64": 1}
# random stream of the walk: the counter-based Philox stream (default) or the
# reference walker's own binary32 MRG recurrence (si_walk_refstream)
RNGS = ("philox", "reference")

SMOOTH_OOM_WARNING = "Warning: GPU out of memory to allocate smooth array. Process continues without smoothing."
UNCERTAINTY_OOM_WARNING = ("Warning: GPU out of memory to allocate uncertainty array. Process continues without "
                           "uncertainty.")


def _or_warn_on_oom(make, warning: str):
    """Returns make(), or None after printing ``warning`` when the device runs
    out of memory: the reference's smoothing and uncertainty steps degrade
    that way instead of failing the job (rw_small.py:147-149, 181-183)."""
    try:
        return make()
    except torch.cuda.OutOfMemoryError:
        print(warning)
        return None


def smooth_tmp_floats(Zc: int, Yc: int, Xc: int) -> int:
    """Floats each si_smooth scratch buffer holds for a (Zc, Yc, Xc) crop."""
    n = ctypes.c_ulonglong(0)
    nat.call("si_smooth_tmp_floats", Zc, Yc, Xc, ctypes.byref(n))
    return int(n.value)


def smooth_buffers(Zc: int, Yc: int, Xc: int, device=None, floats: int = 0):
    """The two float32 scratch buffers of si_smooth / si_smooth_f32 (at least
    ``floats`` each)."""
    n = max(smooth_tmp_floats(Zc, Yc, Xc), int(floats))
    return (torch.empty(n, dtype=torch.float32, device=device), torch.empty(n, dtype=torch.float32, device=device))


def smooth_check():
    """Raises when a smoothing kernel's bounded wait gave up since the last
    check (synchronises the current stream)."""
    st = ctypes.c_int(0)
    nat.call("si_smooth_status", ctypes.byref(st), _stream())


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


_IMG_DTYPES = {np.dtype(np.uint8): nat.SI_U8, np.dtype(np.int8): nat.SI_I8, np.dtype(np.uint16): nat.SI_U16,
               np.dtype(np.int16): nat.SI_I16, np.dtype(np.int32): nat.SI_I32, np.dtype(np.float32): nat.SI_F32}
_LAB_DTYPES = {np.dtype(np.uint8): nat.SI_U8, np.dtype(np.int16): nat.SI_I16, np.dtype(np.int32): nat.SI_I32}
_TORCH = {np.dtype(np.uint8): torch.uint8, np.dtype(np.int8): torch.int8, np.dtype(np.uint16): torch.uint16
          if hasattr(torch, "uint16") else torch.int16, np.dtype(np.int16): torch.int16,
          np.dtype(np.int32): torch.int32, np.dtype(np.float32): torch.float32}


def normalize_host_dtypes(data: np.ndarray, labelData: np.ndarray):
    """Host-side dtype handling done before upload (no O(N) work for the
    common uint8/int32 inputs).

    Image dtypes the device reads directly: uint8, int8, uint16, int16, int32,
    float32; anything else is converted to float32 as numpy's astype does
    (interpolation.py:140-141). Labels: uint8, int16, int32 directly; float
    labels -> int32 (biomedisa_helper.py:665-670); wider integers keep their
    pre-processing meaning (values > 255 become 0, negatives stay ignored)
    before the int32 cast (interpolation.py:145-147)."""
    if np.dtype(data.dtype) not in _IMG_DTYPES:
        data = data.astype(np.float32)
    ld = np.dtype(labelData.dtype)
    if ld in (np.dtype(np.float16), np.dtype(np.float32), np.dtype(np.float64)):
        print(f"Warning: Potential label loss during conversion from {labelData.dtype} to int32.")
        labelData = labelData.astype(np.int32)
    elif ld in (np.dtype(np.int8),):
        labelData = labelData.astype(np.int16)
    elif ld not in _LAB_DTYPES:
        if ld in (np.dtype(np.uint32), np.dtype(np.int64), np.dtype(np.uint64)):
            print(f"Warning: Potential label loss during conversion from {labelData.dtype} to int32.")
        big = labelData > 255
        neg = labelData < 0 if np.issubdtype(ld, np.signedinteger) else None
        lab = labelData.astype(np.int64) if np.issubdtype(ld, np.signedinteger) else labelData
        lab = np.where(big, 0, lab)
        if neg is not None:
            lab = np.where(neg, -1, lab)
        labelData = lab.astype(np.int32)
    return np.ascontiguousarray(data), np.ascontiguousarray(labelData)


@dataclass
class LabelPlan:
    """Host decisions derived from the label histogram (pre_processing)."""

    all_labels: np.ndarray
    nz_lut: np.ndarray      # uint8[256]
    slot_lut: np.ndarray    # int16[256]
    negative_present: bool
    big_present: bool

    @property
    def nol(self) -> int:
        return len(self.all_labels)


def plan_labels(hist: np.ndarray, only: str = "all", ignore: str = "none") -> LabelPlan:
    """pre_processing (biomedisa_helper.py:671-719) from a value histogram:
    hist[0..255] counts of values 0..255, hist[256] negatives, hist[257] > 255."""
    present = [v for v in range(256) if hist[v] > 0]
    if hist[257] > 0:
        print("Warning: Only label values <=255 are allowed. Label values greater than 255 will be removed.")
        if 0 not in present:
            present = [0] + present  # labels > 255 are set to 0
    if hist[256] > 0:
        print("Warning: Negative labels indicate ignored regions.")
    all_labels = list(present)
    removed = set()
    if 0 not in all_labels:
        all_labels = [0] + all_labels
    labels_to_compute = only.split(",")
    if not any(x in ["all", "All", "ALL"] for x in labels_to_compute):
        for k in [k for k in all_labels if str(k) not in labels_to_compute and k > 0]:
            removed.add(k)
            all_labels.remove(k)
    labels_to_remove = ignore.split(",")
    if not any(x in ["none", "None", "NONE"] for x in labels_to_remove):
        for k in labels_to_remove:
            try:
                k = int(k)
            except ValueError:
                continue
            if 0 <= k <= 255:
                removed.add(k)
            if k in all_labels:
                all_labels.remove(k)
    all_labels = np.asarray(all_labels, np.int64)
    slot_of = {int(v): i for i, v in enumerate(all_labels)}
    nz_lut = np.zeros(256, np.uint8)
    slot_lut = np.full(256, -1, np.int16)
    for v in range(256):
        eff = 0 if (v in removed and v != 0) else v
        if v in removed and v == 0:
            eff = 0
        nz_lut[v] = 1 if (eff != 0 and v not in removed) else 0
        slot_lut[v] = slot_of.get(eff, -1)
    return LabelPlan(all_labels, nz_lut, slot_lut, bool(hist[256] > 0), bool(hist[257] > 0))


@dataclass
class CropPlan:
    Z0: int
    Y0: int
    X0: int
    cz0: int
    cy0: int
    cx0: int
    Zc: int
    Yc: int
    Xc: int
    slice_list: np.ndarray  # int32 (n, 2): (axis, index in crop)

    @property
    def crop(self):
        return (self.cz0, self.cy0, self.cx0, self.Zc, self.Yc, self.Xc)

    @property
    def voxels(self) -> int:
        return self.Zc * self.Yc * self.Xc

    def seed_capacity(self, slice_list=None) -> int:
        per = {0: self.Yc * self.Xc, 1: self.Zc * self.Xc, 2: self.Zc * self.Yc}
        sl = self.slice_list if slice_list is None else slice_list
        return int(sum(per[int(a)] for a, _ in sl))

    @property
    def max_rows(self) -> int:
        return max(self.Zc, self.Yc)


def plan_crop(shape0, bbox, flags, allaxis: bool):
    """predict_blocksize (biomedisa_helper.py:1105-1124) on the padded frame and
    the labelled-slice lists in crop coordinates."""
    Z0, Y0, X0 = shape0
    zsh, ysh, xsh = Z0 + 2, Y0 + 2, X0 + 2
    az, bz, ay, by, ax, bx = (int(v) for v in bbox)
    cz0 = az - 100 if az - 100 > 0 else 0
    cz1 = bz + 100 if bz + 100 < zsh else zsh
    cy0 = ay - 100 if ay - 100 > 0 else 0
    cy1 = by + 100 if by + 100 < ysh else ysh
    cx0 = ax - 100 if ax - 100 > 0 else 0
    cx1 = bx + 100 if bx + 100 < xsh else xsh
    entries = []
    offs = (cz0, cy0, cx0)
    lims = (cz1, cy1, cx1)
    for axis in ((0, 1, 2) if allaxis else (0,)):
        for k in np.nonzero(flags[axis])[0]:
            if offs[axis] <= k < lims[axis]:
                entries.append((axis, int(k) - offs[axis]))
    sl = np.asarray(entries, np.int32).reshape(-1, 2)
    return CropPlan(Z0, Y0, X0, cz0, cy0, cx0, cz1 - cz0, cy1 - cy0, cx1 - cx0, sl)


@dataclass
class Timings:
    stages: dict = field(default_factory=dict)

    def mark(self, name, t0):
        self.stages[name] = self.stages.get(name, 0.0) + (time.perf_counter() - t0)


class DeviceJob:
    """One smart interpolation on the current CUDA device. The volumes are
    device tensors (uploaded by the caller or by ``from_host``)."""

    def __init__(self, img: torch.Tensor, img_code: int, lab: torch.Tensor, lab_code: int, *, nbrw=10, sorw=4000,
                 allaxis=False, smooth=0, uncertainty=False, denoise=False, only="all", ignore="none",
                 rng_seed=DEFAULT_RNG_SEED, walk_grid=0, walk_block=0, walk_order=0, walker="auto",
                 sweep_steps=0, sort_edge=0, seeding="plain", rng="philox", smooth_update="f32"):
        if walker not in WALKERS:
            raise ValueError(f"walker must be one of {WALKERS}")
        if seeding not in SEEDINGS:
            raise ValueError(f"seeding must be one of {SEEDINGS}")
        if smooth_update not in SMOOTH_UPDATES:
            raise ValueError(f"smooth_update must be one of {tuple(SMOOTH_UPDATES)}")
        self.smooth_update = smooth_update
        if rng not in RNGS:
            raise ValueError(f"rng must be one of {RNGS}")
        if rng == "reference" and seeding == "large":
            raise ValueError("rng='reference' is supported with the plain seed set only")
        self.rng = rng
        self.seeding = seeding
        self.sweep_steps = int(sweep_steps)
        self.sort_edge = int(sort_edge)
        self.walker = walker
        if img.dim() != 3 or lab.dim() != 3 or tuple(img.shape) != tuple(lab.shape):
            raise ValueError("image and labels must be 3-D volumes of the same shape")
        if not (img.is_cuda and lab.is_cuda) or img.device != lab.device:
            raise ValueError("image and labels must be tensors on one CUDA device")
        self.img, self.img_code, self.lab, self.lab_code = img, img_code, lab, lab_code
        self.shape0 = tuple(int(s) for s in img.shape)
        self.nbrw, self.sorw = int(nbrw), int(sorw)
        self.allaxis, self.smooth, self.uncertainty, self.denoise = bool(allaxis), int(smooth), bool(uncertainty), \
            bool(denoise)
        self.only, self.ignore = only, ignore
        self.rng_seed = int(rng_seed) & 0xFFFFFFFFFFFFFFFF
        self.walk_grid, self.walk_block, self.walk_order = walk_grid, walk_block, walk_order
        self.dev = img.device
        self.launches = 0

    # -- host decisions ----------------------------------------------------
    def analyze(self):
        """Label histogram, label plan, slice flags, bbox and crop plan.
        Returns an error message or None."""
        n = self.img.numel()
        hist = torch.zeros(258, dtype=torch.int64, device=self.dev)
        nat.call("si_label_histogram", _ptr(self.lab), self.lab_code, n, _ptr(hist), _stream())
        self.launches += 1
        h = hist.cpu().numpy()
        self.lplan = plan_labels(h, self.only, self.ignore)
        if self.lplan.nol < 2:
            return "No labeled slices found."
        Z0, Y0, X0 = self.shape0
        fz = torch.zeros(Z0 + 2, dtype=torch.uint8, device=self.dev)
        fy = torch.zeros(Y0 + 2, dtype=torch.uint8, device=self.dev)
        fx = torch.zeros(X0 + 2, dtype=torch.uint8, device=self.dev)
        imax = np.iinfo(np.int32).max
        bbox = torch.tensor([imax, -1, imax, -1, imax, -1], dtype=torch.int32, device=self.dev)
        nz = torch.from_numpy(self.lplan.nz_lut).to(self.dev)
        nat.call("si_slice_flags", _ptr(self.lab), self.lab_code, Z0, Y0, X0, _ptr(nz), int(self.allaxis), _ptr(fz),
                 _ptr(fy), _ptr(fx), _ptr(bbox), _stream())
        self.launches += 1
        flags = [fz.cpu().numpy(), fy.cpu().numpy(), fx.cpu().numpy()]
        bb = bbox.cpu().numpy()
        if bb[1] < 0:
            return "No labeled slices found."
        if self.allaxis:
            for a in range(3):
                k = np.nonzero(flags[a])[0]
                if np.any(np.diff(k) == 1):
                    return "At least one empty slice between labels required."
        self.cplan = plan_crop(self.shape0, bb, flags, self.allaxis)
        return None

    # -- device work -------------------------------------------------------
    def prepare(self):
        """Working image and seeds."""
        cp = self.cplan
        self.work_is_float = self.img_code not in (nat.SI_U8, nat.SI_I8)
        mn, rng = 0.0, 1.0
        if self.work_is_float:
            mm = torch.tensor([np.inf, -np.inf], dtype=torch.float32, device=self.dev)
            nat.call("si_image_minmax", _ptr(self.img), self.img_code, self.img.numel(), _ptr(mm), _stream())
            self.launches += 1
            lo, hi = (np.float32(v) for v in mm.cpu().numpy())
            rng = np.float32(hi - lo)
            if not np.isfinite(rng) or rng == 0:
                raise ValueError("image is constant or not finite; the [0,255] normalisation is undefined")
            mn = lo
        self.work = torch.empty(cp.voxels, dtype=torch.float32 if self.work_is_float else torch.uint8,
                                device=self.dev)
        nat.call("si_prepare_image", _ptr(self.img), self.img_code, *self.shape0, *cp.crop, float(mn), float(rng),
                 int(self.denoise), _ptr(self.work), _stream())
        self.launches += 1
        slice_list = cp.slice_list
        if self.seeding == "large":
            slice_list = large_allx_slice_list(self) if self.allaxis else large_slice_list(cp.slice_list)
        cap = max(cp.seed_capacity(slice_list), 1)
        self.seed_capacity = cap
        self.seeds = torch.empty(cap * SEED_RECORD_BYTES, dtype=torch.uint8, device=self.dev)
        self.n_seeds = torch.zeros(1, dtype=torch.int32, device=self.dev)
        n_sl = len(slice_list)
        self.row_counts = torch.zeros(max(n_sl * cp.max_rows + 1, 1), dtype=torch.int32, device=self.dev)
        sl = torch.from_numpy(np.ascontiguousarray(slice_list.reshape(-1))).to(self.dev) if n_sl else \
            torch.zeros(2, dtype=torch.int32, device=self.dev)
        slot_lut = torch.from_numpy(self.lplan.slot_lut).to(self.dev)
        slot_label = np.zeros(256, np.uint8)
        slot_label[: self.lplan.nol] = self.lplan.all_labels.astype(np.uint8)
        self.slot_label = torch.from_numpy(slot_label).to(self.dev)
        if self.seeding == "large":
            self._large_seeds(slice_list, sl, slot_lut)
        else:
            nat.call("si_extract_seeds", _ptr(self.lab), self.lab_code, *self.shape0, *cp.crop, _ptr(slot_lut),
                     _ptr(self.slot_label), _ptr(self.work), int(self.work_is_float), _ptr(sl), n_sl,
                     _ptr(self.row_counts), _ptr(self.seeds), _ptr(self.n_seeds), _stream())
            self.launches += 3
        long_walks = self.nbrw * self.sorw >= (1 << 24)
        kind = self.walker
        if self.rng == "reference":
            kind = "refstream"  # one thread per seed over packed records
        elif kind == "auto":
            kind = "packed" if long_walks else "sorted"
        if kind == "tiles" and (self.work_is_float or long_walks):
            raise ValueError("the tile walker needs a uint8 volume and nbrw*sorw < 2^24")
        if kind == "sorted" and long_walks:
            raise ValueError("the sorted walker needs nbrw*sorw < 2^24")
        self.walker_used = kind
        if kind != "tiles":
            self.packed = pack_neighbours(self.work, self.work_is_float, cp.Zc, cp.Yc, cp.Xc)
            self.launches += 1

    def _large_seeds(self, slice_list, sl, slot_lut):
        """The reference large path's seed set: taken slices (slice_list),
        labels outside the in-plane box read as ignored, adaptive filter."""
        if self.allaxis:
            return self._large_allx_seeds(slice_list, sl, slot_lut)
        cp = self.cplan
        taken = [int(z) for _, z in slice_list.tolist()]
        self.large_box = large_slice_box(self, taken)
        y0, y1, x0, x1 = self.large_box
        n_sl = len(taken)
        raw = torch.empty_like(self.seeds)
        n_raw = torch.zeros(1, dtype=torch.int32, device=self.dev)
        nat.call("si_extract_seeds_box", _ptr(self.lab), self.lab_code, *self.shape0, *cp.crop, _ptr(slot_lut),
                 _ptr(self.slot_label), _ptr(self.work), int(self.work_is_float), _ptr(sl), n_sl, y0, y1, x0, x1,
                 _ptr(self.row_counts), _ptr(raw), _ptr(n_raw), _stream())
        need = ctypes.c_uint64(0)
        nat.call("si_adaptive_scratch_bytes", cp.Zc, cp.Yc, cp.Xc, n_sl, ctypes.byref(need))
        scratch = torch.empty(max(int(need.value), 1), dtype=torch.uint8, device=self.dev)
        zs = torch.tensor(taken if taken else [0], dtype=torch.int32, device=self.dev)
        nat.call("si_adaptive_seed_filter", _ptr(self.lab), self.lab_code, *self.shape0, *cp.crop, _ptr(slot_lut),
                 _ptr(self.slot_label), _ptr(zs), n_sl, y0, y1, x0, x1, _ptr(raw), _ptr(n_raw), self.seed_capacity,
                 _ptr(self.seeds), _ptr(self.n_seeds), _ptr(scratch), int(need.value), _stream())
        self.launches += 3 + 5

    def _large_allx_seeds(self, slice_list, sl, slot_lut):
        """The all-axis large path's seed set (rw_large.py:68-107 on one GPU,
        pycuda_large_allx.py:309-322): every listed slice, one label box per
        axis (labels outside read as ignored), adaptive filter in each
        slice's own plane."""
        cp = self.cplan
        n_sl = len(slice_list)
        boxes = np.zeros(12, np.int32)
        for axis in range(3):
            idx = [int(k) for a, k in slice_list.tolist() if a == axis]
            boxes[4 * axis:4 * axis + 4] = large_plane_box(self, axis, idx, ignore_minus_one=True)
        self.large_boxes = boxes.reshape(3, 4).copy()
        raw = torch.empty_like(self.seeds)
        n_raw = torch.zeros(1, dtype=torch.int32, device=self.dev)
        nat.call("si_extract_seeds_boxes", _ptr(self.lab), self.lab_code, *self.shape0, *cp.crop, _ptr(slot_lut),
                 _ptr(self.slot_label), _ptr(self.work), int(self.work_is_float), _ptr(sl), n_sl,
                 boxes.ctypes.data, _ptr(self.row_counts), _ptr(raw), _ptr(n_raw), _stream())
        need = ctypes.c_uint64(0)
        nat.call("si_adaptive_scratch_bytes_allx", cp.Zc, cp.Yc, cp.Xc, n_sl, ctypes.byref(need))
        scratch = torch.empty(max(int(need.value), 1), dtype=torch.uint8, device=self.dev)
        nat.call("si_adaptive_seed_filter_allx", _ptr(self.lab), self.lab_code, *self.shape0, *cp.crop,
                 _ptr(slot_lut), _ptr(self.slot_label), _ptr(sl), n_sl, boxes.ctypes.data, _ptr(raw), _ptr(n_raw),
                 self.seed_capacity, _ptr(self.seeds), _ptr(self.n_seeds), _ptr(scratch), int(need.value),
                 _stream())
        self.launches += 3 + 5

    def walk(self):
        cp = self.cplan
        nol = self.lplan.nol
        self.hits = torch.zeros((nol, cp.Zc, cp.Yc, cp.Xc), dtype=torch.int32, device=self.dev)
        if self.walker_used == "tiles":
            self.rounds = walk_bricks(self.work, cp.Zc, cp.Yc, cp.Xc, self.seeds, self.n_seeds, self.seed_capacity,
                                      self.nbrw, self.sorw, self.rng_seed, self.hits, nol)
            self.launches += 1 + 9 * self.rounds
            return
        if self.walker_used == "refstream":
            # the reference's stream: one thread per seed, its walks in sequence;
            # rank of every listed slice among the listed slices of its axis
            rank = np.full(cp.Zc + cp.Yc + cp.Xc, -1, np.int32)
            base = {0: 0, 1: cp.Zc, 2: cp.Zc + cp.Yc}
            count = {0: 0, 1: 0, 2: 0}
            for a, k in cp.slice_list.tolist():
                rank[base[a] + k] = count[a]
                count[a] += 1
            rank_t = torch.from_numpy(rank).to(self.dev)
            nat.call("si_walk_refstream", _ptr(self.packed), int(self.work_is_float), cp.Zc, cp.Yc, cp.Xc,
                     _ptr(self.seeds), _ptr(self.n_seeds), self.seed_capacity, self.nbrw, self.sorw, _ptr(rank_t),
                     _ptr(self.hits), nol, _stream())
            self.launches += 1
            return
        if self.walker_used == "sorted":
            self.rounds = walk_sorted(self.packed, self.work_is_float, cp.Zc, cp.Yc, cp.Xc, self.seeds,
                                      self.n_seeds, self.seed_capacity, self.nbrw, self.sorw, self.rng_seed,
                                      self.hits, nol, self.sweep_steps, self.sort_edge)
            # per sweep: scatter, sweep, round shift and three scan kernels
            # (+ one loop-condition kernel per two sweeps on the device loop)
            self.launches += 6 * self.rounds + (self.rounds + 1) // 2 + 10
            return
        nat.call("si_walk", _ptr(self.packed), int(self.work_is_float), cp.Zc, cp.Yc, cp.Xc, _ptr(self.seeds),
                 _ptr(self.n_seeds), self.seed_capacity, self.nbrw, self.sorw, self.rng_seed, _ptr(self.hits), nol,
                 int(self.walk_grid), int(self.walk_block), int(self.walk_order), _stream())
        self.launches += 1

    def _labels_from(self, maps: torch.Tensor, is_float: bool, want_uq: bool):
        cp = self.cplan
        Z0, Y0, X0 = self.shape0
        out = torch.zeros((Z0, Y0, X0), dtype=torch.uint8, device=self.dev)
        presence = torch.zeros(8, dtype=torch.int32, device=self.dev)
        uq = None
        if want_uq:
            uq = _or_warn_on_oom(lambda: torch.zeros((Z0, Y0, X0), dtype=torch.uint8, device=self.dev),
                                 UNCERTAINTY_OOM_WARNING)
        nat.call("si_argmax", _ptr(maps), int(is_float), self.lplan.nol, cp.Zc, cp.Yc, cp.Xc, cp.cz0, cp.cy0,
                 cp.cx0, Z0, Y0, X0, _ptr(out), _ptr(presence), _ptr(uq), _stream())
        nat.call("si_remap_labels", _ptr(out), cp.Zc, cp.Yc, cp.Xc, cp.cz0, cp.cy0, cp.cx0, Z0, Y0, X0,
                 _ptr(presence), _ptr(self.slot_label), self.lplan.nol, _stream())
        self.launches += 2
        return out, uq

    def hits_full(self) -> torch.Tensor:
        """float32 (nol, Z0, Y0, X0) hit maps in the original frame (rw_small.py:193-197)."""
        cp = self.cplan
        Z0, Y0, X0 = self.shape0
        full = torch.zeros((self.lplan.nol, Z0 + 2, Y0 + 2, X0 + 2), dtype=torch.float32, device=self.dev)
        full[:, cp.cz0:cp.cz0 + cp.Zc, cp.cy0:cp.cy0 + cp.Yc, cp.cx0:cp.cx0 + cp.Xc] = self.hits.float()
        return full[:, 1:-1, 1:-1, 1:-1]

    def post_regular(self, return_hits=False):
        """argmax (+ uncertainty) and optional hit maps; a dict of device tensors."""
        res = {}
        out, uq = self._labels_from(self.hits, False, self.uncertainty)
        res["regular"] = out
        if uq is not None:
            res["uncertainty"] = uq
        if return_hits:
            res["hits"] = self.hits_full().contiguous()
        return res

    def smooth_launch(self, tmp0: torch.Tensor, tmp1: torch.Tensor):
        """Launches the smoothing iterations (in place on the hit maps); only
        kernel launches and memsets on the current stream, so it can be
        graph-captured. tmp0/tmp1: smooth_buffers() of at least this crop."""
        cp = self.cplan
        nat.call("si_smooth", _ptr(self.hits), _ptr(tmp0), _ptr(tmp1), self.lplan.nol, cp.Zc, cp.Yc, cp.Xc,
                 self.smooth, SMOOTH_UPDATES[self.smooth_update], _stream())
        self.launches += self.lplan.nol * (self.smooth + 1 if self.smooth else 1)

    def post_smooth(self):
        if self.seeding == "large":
            # pycuda_large.py:440-444: label 0's smoothed map is clamped at 0
            plane = self.hits[0].view(torch.float32)
            plane.clamp_(min=0.0)
        sm, _ = self._labels_from(self.hits, True, False)
        return sm

    def post(self, return_hits=False):
        """argmax (+uncertainty), optional hits, optional smoothing. Returns a
        dict of device tensors."""
        res = self.post_regular(return_hits)
        if self.smooth:
            cp = self.cplan
            tmp = _or_warn_on_oom(lambda: smooth_buffers(cp.Zc, cp.Yc, cp.Xc, self.dev), SMOOTH_OOM_WARNING)
            if tmp is None:
                self.smooth = 0
            else:
                self.smooth_launch(*tmp)
                smooth_check()
                res["smooth"] = self.post_smooth()
        return res

    def total_steps(self) -> int:
        return int(self.n_seeds.item()) * self.nbrw * self.sorw


def large_slice_list(slice_list: np.ndarray) -> np.ndarray:
    """read_labeled_slices_large (biomedisa_helper.py:1068-1080) on the crop's
    labelled z-slices: after each slice taken, the next four are skipped."""
    out, nxt = [], -1
    for axis, z in slice_list.tolist():
        if axis == 0 and z >= nxt:
            out.append((0, z))
            nxt = z + 5
    return np.asarray(out, np.int32).reshape(-1, 2)


def large_plane_box(job, axis, idx, ignore_minus_one=False) -> tuple[int, int, int, int]:
    """reduceBlocksize on the stack of an axis' slices (crop indices idx):
    the box of the labels other than 0 (and -1 with ignore_minus_one, as
    pycuda_large_allx.py:37-57 zeroes -1 first; pycuda_large.py:39-58 does
    not) of the slices whose such labels are not all in column 0, grown by 100
    and clamped; (r0, r1, c0, c1) in the slice plane's crop coordinates (z-
    slices: rows y, columns x; y-slices: rows z, columns x; x-slices: rows z,
    columns y). Labels outside the box read as -1."""
    cp = job.cplan
    dims_c = (cp.Zc, cp.Yc, cp.Xc)
    offs = (cp.cz0 - 1, cp.cy0 - 1, cp.cx0 - 1)
    dims0 = job.shape0
    ra, ca = {0: (1, 2), 1: (0, 2), 2: (0, 1)}[axis]
    R, C = dims_c[ra], dims_c[ca]
    amin_c, amax_c, amin_r, amax_r = C, 0, R, 0
    orig = [k + offs[axis] for k in idx if 0 <= k + offs[axis] < dims0[axis]]  # pad slices hold no label
    if orig:
        rs, re = max(offs[ra], 0), min(offs[ra] + R, dims0[ra])
        cs, ce = max(offs[ca], 0), min(offs[ca] + C, dims0[ca])
        o = torch.tensor(orig, dtype=torch.int64, device=job.dev)
        v = job.lab.index_select(axis, o).movedim(axis, 0)[:, rs:re, cs:ce].to(torch.int32)
        eff_lut = np.zeros(256, np.int32)
        for k in range(256):
            slot = int(job.lplan.slot_lut[k])
            eff_lut[k] = int(job.lplan.all_labels[slot]) if slot >= 0 else 0
        lut = torch.from_numpy(eff_lut).to(job.dev)
        eff = torch.where(v < 0, v, torch.where(v > 255, torch.zeros_like(v), lut[v.clamp(0, 255).long()]))
        nz = eff != 0
        if ignore_minus_one:
            nz &= eff != -1
        ccoord = torch.arange(cs - offs[ca], ce - offs[ca], device=job.dev)  # crop columns of the loaded ones
        qual = (nz & (ccoord != 0)[None, None, :]).flatten(1).any(1)
        nzq = nz & qual[:, None, None]
        rows = nzq.any(2).any(0)
        cols = nzq.any(1).any(0)
        if bool(rows.any()):
            ry = torch.nonzero(rows).flatten()
            cx = torch.nonzero(cols).flatten()
            amin_r, amax_r = int(ry[0]) + rs - offs[ra], int(ry[-1]) + rs - offs[ra]
            amin_c, amax_c = int(cx[0]) + cs - offs[ca], int(cx[-1]) + cs - offs[ca]
    amin_c = amin_c - 100 if amin_c - 100 > 0 else 0
    amax_c = amax_c + 100 if amax_c + 100 < C else C
    amin_r = amin_r - 100 if amin_r - 100 > 0 else 0
    amax_r = amax_r + 100 if amax_r + 100 < R else R
    return amin_r, amax_r, amin_c, amax_c


def large_slice_box(job, taken) -> tuple[int, int, int, int]:
    """reduceBlocksize (pycuda_large.py:39-58) on the taken z-slices of the
    crop: (y0, y1, x0, x1) in crop coordinates, labels outside read as -1."""
    return large_plane_box(job, 0, taken)


def large_allx_slice_list(job) -> np.ndarray:
    """The all-axis large path's slices (rw_large.py:68-107, one GPU): for
    each axis the slices of the crop that keep a positive label after the
    one-pixel-line removal (read_labeled_slices_allx_large,
    biomedisa_helper.py:1082-1099; no skipping); (axis, crop index) pairs,
    z-slices first."""
    cp = job.cplan
    Z0, Y0, X0 = job.shape0
    fz = torch.zeros(Z0 + 2, dtype=torch.uint8, device=job.dev)
    fy = torch.zeros(Y0 + 2, dtype=torch.uint8, device=job.dev)
    fx = torch.zeros(X0 + 2, dtype=torch.uint8, device=job.dev)
    imax = np.iinfo(np.int32).max
    bbox = torch.tensor([imax, -1, imax, -1, imax, -1], dtype=torch.int32, device=job.dev)
    nz = torch.from_numpy(job.lplan.nz_lut).to(job.dev)
    nat.call("si_slice_flags", _ptr(job.lab), job.lab_code, Z0, Y0, X0, _ptr(nz), 2, _ptr(fz), _ptr(fy), _ptr(fx),
             _ptr(bbox), _stream())
    job.launches += 1
    flags = [f.cpu().numpy() for f in (fz, fy, fx)]
    offs = (cp.cz0, cp.cy0, cp.cx0)
    lims = (cp.cz0 + cp.Zc, cp.cy0 + cp.Yc, cp.cx0 + cp.Xc)
    out = [(a, int(k) - offs[a]) for a in range(3) for k in np.nonzero(flags[a])[0] if offs[a] <= k < lims[a]]
    return np.asarray(out, np.int32).reshape(-1, 2)


def pack_neighbours(work: torch.Tensor, is_float: bool, Zc: int, Yc: int, Xc: int) -> torch.Tensor:
    """Packed neighbourhood records of a working volume (si_pack_neighbours)."""
    rec = 32 if is_float else 8
    packed = torch.empty(Zc * Yc * Xc * rec, dtype=torch.uint8, device=work.device)
    nat.call("si_pack_neighbours", _ptr(work), int(is_float), Zc, Yc, Xc, _ptr(packed), _stream())
    return packed


def walk_bricks(work, Zc, Yc, Xc, seeds, n_seeds, max_seeds, nbrw, sorw, key, hits, nol) -> int:
    """Brick walker (si_walk_bricks) with scratch from the caching allocator.
    Returns the number of rounds."""
    need = ctypes.c_ulonglong(0)
    walks = int(max_seeds) * int(nbrw)
    nat.call("si_walk_bricks_scratch", Zc, Yc, Xc, walks, nol, ctypes.byref(need))
    scratch = torch.empty(max(int(need.value), 1), dtype=torch.uint8, device=work.device)
    rounds = ctypes.c_int(0)
    nat.call("si_walk_bricks", _ptr(work), Zc, Yc, Xc, _ptr(seeds), _ptr(n_seeds), int(max_seeds), int(nbrw),
             int(sorw), int(key), _ptr(hits), nol, _ptr(scratch), int(need.value), ctypes.byref(rounds), _stream())
    return int(rounds.value)


def walk_sorted(packed, is_float, Zc, Yc, Xc, seeds, n_seeds, max_seeds, nbrw, sorw, key, hits, nol,
                sweep_steps=0, sort_edge=0) -> int:
    """Sorted-sweep walker (si_walk_sorted) with scratch from the caching
    allocator. Returns the number of sweeps."""
    need = ctypes.c_ulonglong(0)
    nat.call("si_walk_sorted_scratch", Zc, Yc, Xc, int(max_seeds) * int(nbrw), nol, int(sort_edge),
             ctypes.byref(need))
    scratch = torch.empty(max(int(need.value), 1), dtype=torch.uint8, device=packed.device)
    rounds = ctypes.c_int(0)
    nat.call("si_walk_sorted", _ptr(packed), int(is_float), Zc, Yc, Xc, _ptr(seeds), _ptr(n_seeds), int(max_seeds),
             int(nbrw), int(sorw), int(key), _ptr(hits), nol, int(sweep_steps), int(sort_edge), _ptr(scratch),
             int(need.value),
             ctypes.byref(rounds), _stream())
    return int(rounds.value)


def upload(data: np.ndarray, labelData: np.ndarray, device=None, pinned=True):
    """Copies host volumes to the device (pinned staging for full H2D speed)."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    tens = []
    for arr in (data, labelData):
        t = torch.from_numpy(arr.view(np.int16) if arr.dtype == np.uint16 and not hasattr(torch, "uint16") else arr)
        if pinned:
            t = t.pin_memory()
        tens.append(t.to(dev, non_blocking=pinned))
    return tens[0], tens[1]


def smart_interpolation(data, labelData, nbrw=10, sorw=4000, acwe=False, acwe_alpha=1.0, acwe_smooth=1,
                        acwe_steps=3, path_to_data=None, path_to_labels=None, denoise=False, uncertainty=False,
                        platform=None, allaxis=False, ignore="none", only="all", smooth=0, compression=True,
                        return_hits=False, img_id=None, label_id=None, remote=False, queue=0, clean=None, fill=None,
                        slicer=False, *, rng_seed=DEFAULT_RNG_SEED, device=None, return_device=False,
                        walk_grid=0, walk_block=0, walk_order=0, walker="auto", sweep_steps=0, sort_edge=0,
                        seeding="plain", rng="philox", smooth_update="f32"):
    """Smart interpolation of sparsely pre-segmented slices on one GB300.

    Same parameters and result keys as the reference
    (biomedisa/interpolation.py:43-46; results 'regular' and, when asked,
    'smooth', 'uncertainty', 'hits', and with ``clean`` / ``fill`` thresholds
    'cleaned', 'smooth_cleaned', 'filled', 'cleaned_filled' as
    rw_small.py:223-243). Errors print 'Error: ...' and return
    None as the reference does. ``platform`` is accepted and ignored (one CUDA
    device). Extra keyword-only arguments: ``rng_seed`` (Philox key),
    ``device``, ``return_device`` (keep results as device tensors), ``walker``
    ('auto' = 'sorted': sorted sweeps of ``sweep_steps`` steps over bricks of
    ``sort_edge``^3 voxels (0 = library defaults); 'tiles':
    shared-memory brick walker, uint8 only; 'packed': one thread per walk) and
    the packed walker's launch shape (``walk_grid``, ``walk_block``,
    ``walk_order``). All walkers give identical hit maps. ``seeding='large'``
    walks the seed set of the reference's large path (z-slices: slice
    skipping, label box, adaptive seeds; all-axis: every slice with a positive
    label, a label box per axis, adaptive seeds in each slice's plane) instead
    of every seed. ``acwe=True`` adds 'acwe' and 'refined' (the reference's
    activeContour on the regular result, rw_small.py:246-255).
    ``rng``: the walk's random stream — 'philox' (counter-based Philox4x32-10
    keyed by ``rng_seed``, the default) or 'reference' (the reference walker's
    own binary32 MRG recurrence, seeded per seed as its CUDA kernel does,
    pycuda_small.py:155-225; one thread per seed, slower), which reproduces
    the reference's own labels up to the last bits of the exp weights.
    ``smooth_update``: arithmetic of the smoothing update phi + 0.01 * kappa —
    'f32' (binary32, the default) or 'ref_f64' (the reference's binary64
    product and sum, gpu_kernels.py:133, rounded to binary32 on the store).
    """
    if data is None or labelData is None:
        raise NotImplementedError("loading volumes from files is outside this package; pass numpy arrays")
    if not torch.cuda.is_available():
        raise RuntimeError("smart_interpolation needs a CUDA device; there is no CPU fallback")
    data = np.asarray(data)
    labelData = np.asarray(labelData)
    if labelData.ndim != 3:
        return _err("Label data must be three-dimensional.")
    if data.shape != labelData.shape:
        return _err("Image and label data must have the same x,y,z-dimensions.")
    data, labelData = normalize_host_dtypes(data, labelData)
    img, lab = upload(data, labelData, device)
    job = DeviceJob(img, _IMG_DTYPES[np.dtype(data.dtype)], lab, _LAB_DTYPES[np.dtype(labelData.dtype)], nbrw=nbrw,
                    sorw=sorw, allaxis=allaxis, smooth=smooth, uncertainty=uncertainty, denoise=denoise, only=only,
                    ignore=ignore, rng_seed=rng_seed, walk_grid=walk_grid, walk_block=walk_block,
                    walk_order=walk_order, walker=walker, sweep_steps=sweep_steps, sort_edge=sort_edge,
                    seeding=seeding, rng=rng, smooth_update=smooth_update)
    msg = job.analyze()
    if msg:
        return _err(msg)
    job.prepare()
    job.walk()
    res = job.post(return_hits=return_hits)
    if clean or fill:
        from .postprocess import post_results

        post_results(res, clean, fill)
    if acwe:
        # rw_small.py:246-252: both activeContour calls on the working image
        # (zero outside the crop) and the regular result
        from .active_contour import Frame, acwe_results

        cp = job.cplan
        frame = Frame(job.work, nat.SI_F32 if job.work_is_float else nat.SI_U8, (cp.cz0, cp.cy0, cp.cx0),
                      (cp.Zc, cp.Yc, cp.Xc))
        res["acwe"], res["refined"] = acwe_results(frame, res["regular"], acwe_alpha, acwe_smooth, acwe_steps)
    # sanity check of rw_small.py:203-211 (Dice of the input slices vs result)
    mask = lab > 0
    gt = lab.to(torch.int32)
    rr = res["regular"].to(torch.int32) * mask
    den = float((gt > 0).sum() + (rr > 0).sum())
    dice = 2.0 * float(torch.logical_and(gt == rr, (gt + rr) > 0).sum()) / den if den else 1.0
    if dice < 0.3:
        print('Warning: Bad result! Use "--allaxis" if you labeled axes other than the xy-plane.')
    if return_device:
        return res
    return {k: (v.cpu().numpy() if v is not None else None) for k, v in res.items()}


def walk(data, slices, indices, indices_child, nbrw, sorw, name=None, ctx=None, queue=None, allx=False,
         rng_seed=DEFAULT_RNG_SEED):
    """Plugin seam of the reference's walkers (pycuda_small.py:35-57,
    pycuda_small_allx.py:35-73, pyopencl_small.py:33-68).

    data: cropped padded volume (uint8 or float32); slices: label slice stack
    (allx: list of three stacks); indices: slice positions (allx: (k, axis)
    pairs); indices_child: the subset of indices this call walks.
    Returns float32 hit maps [labels][z][y][x] for the non-negative labels
    present in ``slices``, as the reference walkers do."""
    if not torch.cuda.is_available():
        raise RuntimeError("walk needs a CUDA device; there is no CPU fallback")
    data = np.ascontiguousarray(data)
    Z, Y, X = data.shape
    vol = np.zeros((Z, Y, X), np.int32)
    entries = []
    if allx:
        stacks = list(slices)
        labels = np.unique(np.concatenate([np.unique(s) for s in stacks]))
        for axis in range(3):
            idx = [k for (k, a) in indices if a == axis]
            child = {k for (k, a) in indices_child if a == axis}
            for j, k in enumerate(idx):
                if k not in child:
                    continue
                if axis == 0:
                    vol[k] = stacks[0][j]
                elif axis == 1:
                    vol[:, k, :] = stacks[1][j]
                else:
                    vol[:, :, k] = stacks[2][j]
                entries.append((axis, k))
    else:
        labels = np.unique(slices)
        child = set(indices_child)
        for j, k in enumerate(indices):
            if k in child:
                vol[k] = slices[j]
                entries.append((0, k))
    labels = labels[labels >= 0].astype(np.int64)
    if data.dtype != np.uint8:
        data = data.astype(np.float32)
    slot_lut = np.full(256, -1, np.int16)
    for i, v in enumerate(labels):
        if 0 <= v <= 255:
            slot_lut[v] = i
    nol = len(labels)
    dev = torch.device("cuda", torch.cuda.current_device())
    img_t = torch.from_numpy(data).to(dev)
    lab_t = torch.from_numpy(vol).to(dev)
    slot_label = np.zeros(256, np.uint8)
    slot_label[:nol] = labels.astype(np.uint8)
    cp = CropPlan(Z, Y, X, 1, 1, 1, Z, Y, X, np.asarray(entries, np.int32).reshape(-1, 2))
    cap = max(cp.seed_capacity(), 1)
    seeds = torch.empty(cap * SEED_RECORD_BYTES, dtype=torch.uint8, device=dev)
    n_seeds = torch.zeros(1, dtype=torch.int32, device=dev)
    rows = torch.zeros(max(len(entries) * cp.max_rows + 1, 1), dtype=torch.int32, device=dev)
    sl = torch.from_numpy(np.ascontiguousarray(cp.slice_list.reshape(-1))).to(dev) if entries else \
        torch.zeros(2, dtype=torch.int32, device=dev)
    is_float = data.dtype == np.float32
    # device copies must stay referenced until the kernels have run: a freed
    # block can be handed to the next allocation on the same stream
    slot_lut_t = torch.from_numpy(slot_lut).to(dev)
    slot_label_t = torch.from_numpy(slot_label).to(dev)
    nat.call("si_extract_seeds", _ptr(lab_t), nat.SI_I32, Z, Y, X, 1, 1, 1, Z, Y, X, _ptr(slot_lut_t),
             _ptr(slot_label_t), _ptr(img_t), int(is_float), _ptr(sl), len(entries), _ptr(rows), _ptr(seeds),
             _ptr(n_seeds), _stream())
    hits = torch.zeros((max(nol, 1), Z, Y, X), dtype=torch.int32, device=dev)
    packed = pack_neighbours(img_t, is_float, Z, Y, X)
    if int(nbrw) * int(sorw) < (1 << 24):
        walk_sorted(packed, is_float, Z, Y, X, seeds, n_seeds, cap, int(nbrw), int(sorw), int(rng_seed), hits,
                    max(nol, 1))
    else:
        nat.call("si_walk", _ptr(packed), int(is_float), Z, Y, X, _ptr(seeds), _ptr(n_seeds), cap, int(nbrw),
                 int(sorw), int(rng_seed), _ptr(hits), max(nol, 1), 0, 0, 0, _stream())
    return hits[:nol].float().cpu().numpy()
