"""Benchmark of the smart-interpolation path on one GB300 (or N replicas).

A step is one complete smart interpolation of the all-axis workload —
uint8 (z, y, x) = (400, 512, 512), 8 phases, labels 0..8 on every 8th XY and
every 16th YZ/XZ slice, nbrw=10, sorw=4000, smooth=100 — on device-resident
inputs: label analysis, working image, seed extraction, the walk, argmax,
100 smoothing iterations per label and the smoothed argmax.

Other workloads (--workload): plain (128^3), screw (419x492x462, the shape and
labelling of the reference's published timing case), large (1024^3), large_ref
(1024^3 with the reference large path's seed set), batch (32 uneven uint16
volumes in one batched walk), train (surrogate training voxels/s), hybrid
(surrogate + restricted walk vs the plain walk at 1024^3, voxels/s), geodesic
(geodesic raster-scan interpolation of the plain volume, voxels/s), acwe (the
active-contour post-processing, voxels/s), conv16 (the surrogate's 16->16
convolution on the tensor cores alone, voxels/s).

Metric: walker-steps/s = (seeds * nbrw * sorw) / step time (whole job).
``e2e`` is the same metric through ``smart_interpolation`` with numpy inputs
and outputs (host->device copies and result download inside the timed region).
``roofline`` covers the walker kernel (the dominant kernel).
``--impl reference`` times the reference's own CPU walker on the host cores.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                       [--workload allaxis|plain|screw|batch|large|large_ref|train|hybrid|geodesic|acwe|conv16]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "allaxis": dict(desc="allaxis uint8 (z,y,x)=(400,512,512), 8 phases, labels every 8th XY + every 16th YZ/XZ "
                         "slice, nbrw=10, sorw=4000, smooth=100", nbrw=10, sorw=4000, smooth=100, allaxis=True),
    "plain": dict(desc="plain uint8 128^3, 2 ellipsoids, labels every 10th z-slice, nbrw=10, sorw=4000, smooth=0",
                  nbrw=10, sorw=4000, smooth=0, allaxis=False),
    "batch": dict(desc="batch of 32 uint16 volumes, sizes uniform in 64^3..(256,320,384) (z,y,x), 2-12 phases, "
                       "labels every 4..20th z-slice, nbrw=10, sorw=4000, smooth=50; one batched walk, smoothing "
                       "replayed from a CUDA graph, autotuned sweep parameters", nbrw=10, sorw=4000, smooth=50,
                  allaxis=False),
    "acwe": dict(desc="activeContour on a uint8 (z,y,x)=(256,384,384) volume of 3 noisy ellipsoids and a "
                      "segmentation of them with jittered borders: both modes as smart_interpolation(acwe=True) runs "
                      "them ('acwe' with alpha=1, smooth=1, steps=3, and 'refined')", nbrw=0, sorw=0, smooth=0,
                 allaxis=False),
    "large": dict(desc="large uint8 1024^3, 6 phases, labels every 12th z-slice, nbrw=10, sorw=4000, smooth=100",
                  nbrw=10, sorw=4000, smooth=100, allaxis=False),
    "screw": dict(desc="screw-like uint8 (z,y,x)=(419,492,462), 2 objects labelled every 20th z-slice, nbrw=10, "
                       "sorw=4000, smooth=0: the dimensions and labelling of the reference's published end-to-end "
                       "timing case (synthetic content)", nbrw=10, sorw=4000, smooth=0, allaxis=False),
    "large_ref": dict(desc="large uint8 1024^3, 6 phases, labels every 12th z-slice, nbrw=10, sorw=4000, "
                           "smooth=100, with the reference large path's seed set (every 5th labelled slice at "
                           "most, label box, adaptive seeds), the configuration the reference itself runs at this "
                           "size", nbrw=10, sorw=4000, smooth=100, allaxis=False, seeding="large"),
    "train": dict(desc="surrogate training: residual 3-D CNN (16 channels, dilations 1,2,4,8, 70 k parameters), "
                       "bf16 activations/weights with fp32 accumulation, batch 8 windows of 64^3 from 16 walked "
                       "128^3 volumes (procedural and large-style), soft-target cross entropy, AdamW",
                  nbrw=10, sorw=4000, smooth=0, allaxis=False),
    "conv16": dict(desc="the surrogate's 16->16 3x3x3 convolution (dilation 1, bias, residual and ReLU, bf16 in "
                        "and out, fp32 accumulation) of a (n,z,y,x) = (1,128,256,1024) bf16 volume (1 GiB per "
                        "activation) on the tcgen05 kernel; the mma.sync kernel timed beside it on the same input",
                   nbrw=0, sorw=0, smooth=0, allaxis=False),
    "hybrid": dict(desc="hybrid vs plain on the large uint8 1024^3 volume (6 phases, labels every 12th z-slice, "
                        "nbrw=10, sorw=4000, smooth=100 in both arms): surrogate everywhere, walk from the seeds "
                        "within 8 voxels of voxels with max p < 0.9 (grown by 2), then 100 smoothing iterations; "
                        "yardstick = the full plain walk with the same smoothing",
                   nbrw=10, sorw=4000, smooth=100, allaxis=False, threshold=0.9, radius=8, coarse=4, grow=2),
    "hybrid_097": dict(desc="as hybrid, with the tighter uncertainty threshold max p < 0.97",
                       nbrw=10, sorw=4000, smooth=100, allaxis=False, threshold=0.97, radius=8, coarse=4, grow=2),
    "geodesic": dict(desc="geodesic interpolation (geodis.geodesic_segment: lamb=1.0, 4 forward+backward raster "
                          "iterations per label) of the plain uint8 128^3 volume, labels 0..2 on every 10th z-slice",
                     nbrw=0, sorw=0, smooth=0, allaxis=False),
}

# one kernel per entry-point call except these (launches per call)
MULTI_LAUNCH = {"si_extract_seeds": 3, "si_nn_conv3d_wgrad": 2}

WALK_SECTORS_L2 = 2  # per walker step at L2: one packed-record sector + one atomic sector
WALK_BYTES_PAYLOAD_U8 = 10  # 6 neighbour bytes + one 4-byte hit per step


def make_batch_inputs(seed: int = 0, count: int = 32):
    from biomedisa_gb300 import synthetic as S

    cache = Path(os.environ.get("SI_BENCH_CACHE", "/tmp")) / f"si_bench_batch_{seed}_{count}.npz"
    if cache.exists():
        z = np.load(cache)
        return [z[f"img{i}"] for i in range(count)], [z[f"lab{i}"] for i in range(count)]
    vols = S.batch_volumes(seed=seed, count=count)
    imgs, labs = [v[0] for v in vols], [v[1] for v in vols]
    try:
        np.savez(cache, **{f"img{i}": a for i, a in enumerate(imgs)}, **{f"lab{i}": a for i, a in enumerate(labs)})
    except OSError:
        pass
    return imgs, labs


def make_inputs(name: str, seed: int = 0):
    from biomedisa_gb300 import synthetic as S

    if name in ("large_ref", "hybrid", "hybrid_097"):
        name = "large"
    if name == "geodesic":
        name = "plain"
    cache = Path(os.environ.get("SI_BENCH_CACHE", "/tmp")) / f"si_bench_{name}_{seed}.npz"
    if cache.exists():
        z = np.load(cache)
        return z["img"], z["lab"]
    if name == "allaxis":
        img, lab, _ = S.allaxis_volume(seed=seed)
    elif name == "plain":
        img, lab, _ = S.plain_volume(seed=seed)
    elif name == "screw":
        img, lab, _ = S.screw_like_volume(seed=seed)
    else:  # large, large_ref, hybrid
        img, lab, _ = S.large_volume(seed=seed)
    try:
        np.savez(cache, img=img, lab=lab)
    except OSError:
        pass
    return img, lab


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.lines: list[str] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, v):
    """Largest value over the ranks (the step time that counts)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def flush_l2(buf):
    buf.add_(1)


def run_job(img_t, img_code, lab_t, lab_code, wl, events=None):
    from biomedisa_gb300.interpolation import DeviceJob

    job = DeviceJob(img_t, img_code, lab_t, lab_code, nbrw=wl["nbrw"], sorw=wl["sorw"], allaxis=wl["allaxis"],
                    smooth=wl["smooth"], seeding=wl.get("seeding", "plain"))
    msg = job.analyze()
    if msg:
        raise RuntimeError(msg)
    job.prepare()
    if events:
        events[0].record()
    job.walk()
    if events:
        events[1].record()
    res = job.post()
    return job, res


def reference_seed_count(lab):
    """Seeds the reference walks for a z-slice-labelled volume: interior
    voxels of the labelled slices of its crop whose label is walked
    (oracle restatement of pre_processing, predict_blocksize and
    read_labeled_slices)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    labelData, all_labels = oracle.pre_processing(lab)
    labelData = np.pad(labelData, 1)
    az, bz, ay, by, ax, bx = oracle.predict_blocksize(labelData)
    labc = labelData[az:bz, ay:by, ax:bx]
    zs = oracle.read_labeled_slices(labc)[0]
    walked = np.zeros(256 + 1, bool)
    walked[np.asarray(all_labels, np.int64)] = True
    n = 0
    for z in zs:
        v = labc[z, 1:-1, 1:-1].astype(np.int64)
        n += int(walked[np.clip(v, 0, 256)][(v >= 0) & (v <= 255)].sum())
    return n


def cpu_baseline(img, lab, wl, target_seconds):
    """The reference's OpenCL walker compiled as C on a bounded sample of this
    workload (same crop/working image the reference would walk)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    import ref_baseline

    labelData, all_labels = oracle.pre_processing(lab)
    data = np.pad(oracle.normalize_image(img), 1)
    labelData = np.pad(labelData, 1)
    az, bz, ay, by, ax, bx = oracle.predict_blocksize(labelData)
    data = np.ascontiguousarray(data[az:bz, ay:by, ax:bx])
    labc = np.ascontiguousarray(labelData[az:bz, ay:by, ax:bx])
    zs = oracle.read_labeled_slices(labc)[0] if not wl["allaxis"] else \
        [k for k, _ in oracle.read_indices_allx(labc, 0)]
    z = zs[len(zs) // 2]
    try:
        return ref_baseline.bounded_sample(data, labc, all_labels, z, wl["nbrw"], wl["sorw"], target_seconds)
    except FileNotFoundError:  # oracle/_ref not built on this host: the oracle's restatement of that kernel
        return ref_baseline.bounded_sample_port(data, labc, all_labels, z, wl["nbrw"], wl["sorw"], target_seconds)


def run_reference(args, wl):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    img, lab = make_inputs(args.workload)
    vals = []
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(img, lab, wl, args.ref_seconds)
        if i >= args.warmup:
            vals.append(cb)
    v = statistics.median(c["value"] for c in vals)
    secs = sum(c["seconds"] for c in vals) / len(vals)
    line = {
        "metric": "walker-steps/s", "value": v, "unit": "walker-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": wl["desc"], "global_batch": 1, "parallelism": "host cores"},
        "cpu_baseline": {"value": v, "unit": "walker-steps/s", "cores": vals[-1]["cores"], "kind": vals[-1]["kind"],
                         "sample": vals[-1]["sample"]},
        "e2e": {"value": v, "unit": "walker-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="allaxis", choices=sorted(WORKLOADS))
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-jobs", type=int, default=0,
                    help="run this many untimed jobs and exit (for ncu captures; no JSON line)")
    ap.add_argument("--nbrw", type=int, default=None, help="override (profiling only)")
    ap.add_argument("--sorw", type=int, default=None, help="override (profiling only)")
    ap.add_argument("--smooth", type=int, default=None, help="override (profiling only)")
    ap.add_argument("--host-loop", action="store_true",
                    help="profiling only: run the walker's sweep loop from the host (same kernels, one launch per "
                         "sweep) so that a profiler sees the kernels the device-side loop runs inside a graph")
    args = ap.parse_args()
    wl = dict(WORKLOADS[args.workload])
    for k in ("nbrw", "sorw", "smooth"):
        if getattr(args, k) is not None:
            if not args.profile_jobs:
                ap.error(f"--{k} is only allowed with --profile-jobs")
            wl[k] = getattr(args, k)
    if args.host_loop and not args.profile_jobs:
        ap.error("--host-loop is only allowed with --profile-jobs")
    if args.profile_jobs:
        profile_jobs(args, wl)
        return
    if args.workload == "batch":
        run_batch_bench(args, wl)
        return
    if args.workload == "train":
        run_train_bench(args, wl)
        return
    if args.workload in ("hybrid", "hybrid_097"):
        run_hybrid_bench(args, wl)
        return
    if args.workload == "conv16":
        run_conv16_bench(args, wl)
        return
    if args.workload == "geodesic":
        run_geodesic_bench(args, wl)
        return
    if args.workload == "acwe":
        run_acwe_bench(args, wl)
        return
    if args.impl == "reference":
        run_reference(args, wl)
        return

    import torch

    from biomedisa_gb300 import interpolation as I
    from biomedisa_gb300 import smart_interpolation

    world, rank, local = dist_setup()
    img, lab = make_inputs(args.workload)
    data, labels = I.normalize_host_dtypes(img, lab)
    img_code, lab_code = I._IMG_DTYPES[data.dtype], I._LAB_DTYPES[labels.dtype]
    img_t, lab_t = I.upload(data, labels)
    torch.cuda.synchronize()
    l2buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    for _ in range(args.warmup):
        run_job(img_t, img_code, lab_t, lab_code, wl)
    torch.cuda.synchronize()

    stream = torch.cuda.current_stream()
    t_steps, t_walk, launches, steps_per_job = [], [], 0, 0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush_l2(l2buf)
            torch.cuda.synchronize()
            barrier(world)
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            ev[2].record(stream)
            job, _ = run_job(img_t, img_code, lab_t, lab_code, wl, events=ev[:2])
            ev[3].record(stream)
            torch.cuda.synchronize()
            barrier(world)
            t_steps.append(ev[2].elapsed_time(ev[3]))
            t_walk.append(ev[0].elapsed_time(ev[1]))
            launches += job.launches
            steps_per_job = job.total_steps()
    ms = max_over_ranks(world, sum(t_steps) / len(t_steps))
    value = world * steps_per_job / (ms / 1e3)
    walk_ms = sum(t_walk) / len(t_walk)
    walk_rate = steps_per_job / (walk_ms / 1e3)

    # end to end through the public API (host numpy in, numpy out)
    e2e_steps = args.e2e_steps or args.steps
    seeding = wl.get("seeding", "plain")
    smart_interpolation(img, lab, nbrw=wl["nbrw"], sorw=wl["sorw"], allaxis=wl["allaxis"], smooth=wl["smooth"],
                        seeding=seeding)
    torch.cuda.synchronize()
    t_e2e = []
    out_bytes = 0
    for _ in range(e2e_steps):
        flush_l2(l2buf)
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        r = smart_interpolation(img, lab, nbrw=wl["nbrw"], sorw=wl["sorw"], allaxis=wl["allaxis"],
                                smooth=wl["smooth"], seeding=seeding)
        torch.cuda.synchronize()
        t_e2e.append(time.perf_counter() - t0)
        out_bytes = sum(v.nbytes for v in r.values())
    e2e_s = max_over_ranks(world, sum(t_e2e) / len(t_e2e))
    e2e_value = world * steps_per_job / e2e_s

    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    peak_kind = "measured" if "hbm_gbs" in peaks else "fallback"
    l2 = measure_l2(torch)
    l2_gbs = l2["read_gbs"]
    achieved_payload = walk_rate * WALK_BYTES_PAYLOAD_U8 / 1e9
    achieved_l2 = walk_rate * WALK_SECTORS_L2 * 32 / 1e9
    traffic, traffic_per_step = None, None
    sweeps = max(getattr(job, "rounds", 0) or 0, 1)
    tp = ROOT / "profiles" / "walker_traffic.json"
    if tp.exists():
        tj = json.loads(tp.read_text())
        if tj.get("workload") == args.workload:
            traffic_per_step = tj["dram_bytes_per_step"]
            traffic = traffic_per_step * steps_per_job / sweeps  # DRAM bytes per sweep launch

    line = {
        "metric": "walker-steps/s", "value": value, "unit": "walker-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded generator, no public dataset)",
        "config": {"workload": wl["desc"], "global_batch": 1, "parallelism": f"replicas x{world}" if world > 1
                   else "single GPU", "l2": "256 MiB buffer written before every timed step; hit maps 3.8 GB > L2"},
        "voxels_per_s": world * int(np.prod(img.shape)) / (ms / 1e3),
        "walk_ms": walk_ms, "walk_steps_per_s": walk_rate, "total_walker_steps": steps_per_job,
        "e2e": {"value": e2e_value, "unit": "walker-steps/s", "seconds": e2e_s,
                "h2d_bytes_per_step": int(img.nbytes + lab.nbytes), "d2h_bytes_per_step": int(out_bytes)},
        "gpu_launches": launches // max(args.steps, 1),
        "roofline": {"bound": "l2", "achieved": achieved_l2, "peak": l2_gbs, "unit": "GB/s",
                     "frac": achieved_l2 / l2_gbs if l2_gbs else None, "traffic": traffic,
                     "atomics_per_s": walk_rate, "atomic_peak_per_s": l2["atomics_per_s"],
                     "atomic_frac": walk_rate / l2["atomics_per_s"] if l2.get("atomics_per_s") else None,
                     "note": f"walker (sorted-sweep kernel, two walkers per thread, {sweeps} sweeps per job on "
                             "the device-side loop), issue- and L2-bound: "
                             f"{WALK_SECTORS_L2} x 32 B sectors per step at L2 (one packed neighbourhood record "
                             "+ one hit atomic) x steps / CUDA-event walk duration; peak = L2 read ceiling "
                             "measured in this run by si_probe_l2_read over a 48 MiB L2-resident buffer (no L2 "
                             "figure in the measured-peaks file); atomic peak = si_probe_l2_atomics; traffic = "
                             f"DRAM bytes per sweep launch from the committed ncu summary ({traffic_per_step} "
                             "B/step, scaled by steps per launch)"},
        "roofline_hbm": {"bound": "hbm", "achieved": achieved_payload, "peak": hbm, "unit": "GB/s",
                         "frac": achieved_payload / hbm,
                         "note": f"walker logical payload {WALK_BYTES_PAYLOAD_U8} B/step (6 neighbour bytes + "
                                 f"4-byte hit) against HBM; peak {peak_kind} (hbm_gbs)"},
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = {k: v for k, v in cpu_baseline(img, lab, wl, args.ref_seconds).items()
                                    if k in ("value", "unit", "cores", "kind", "sample")}
        except Exception as e:  # baseline unavailable must not hide the GPU number
            line["cpu_baseline"] = {"value": None, "unit": "walker-steps/s", "cores": 0, "kind": "reference",
                                    "sample": f"unavailable: {e}"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_batch_bench(args, wl):
    """Batched workload: value = walker steps of all volumes / batch time on
    device-resident volumes; e2e through smart_interpolation_batch."""
    import torch

    from biomedisa_gb300 import interpolation as I
    from biomedisa_gb300 import smart_interpolation_batch
    from biomedisa_gb300.batch import run_device_batch

    world, rank, local = dist_setup()
    imgs, labs = make_batch_inputs()
    dev = []
    for img, lab in zip(imgs, labs):
        d, l = I.normalize_host_dtypes(img, lab)
        ti, tl = I.upload(d, l)
        dev.append((ti, I._IMG_DTYPES[d.dtype], tl, I._LAB_DTYPES[l.dtype]))
    torch.cuda.synchronize()
    l2buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    kw = dict(nbrw=wl["nbrw"], sorw=wl["sorw"], smooth=wl["smooth"])
    for _ in range(args.warmup):
        run_device_batch(dev, **kw)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    times, steps, rep = [], 0, {}
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush_l2(l2buf)
            torch.cuda.synchronize()
            barrier(world)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            jobs, res, rep = run_device_batch(dev, **kw)
            e.record(stream)
            torch.cuda.synchronize()
            barrier(world)
            times.append(s.elapsed_time(e))
            steps = rep["walker_steps"]
    ms = max_over_ranks(world, sum(times) / len(times))
    value = world * steps / (ms / 1e3)
    t_e2e = []
    for _ in range(args.e2e_steps or args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = smart_interpolation_batch(imgs, labs, **kw)
        torch.cuda.synchronize()
        t_e2e.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(world, sum(t_e2e) / len(t_e2e))
    line = {
        "metric": "walker-steps/s", "value": value, "unit": "walker-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded generator, no public dataset)",
        "config": {"workload": wl["desc"], "global_batch": len(imgs), "parallelism": "single GPU",
                   "l2": "256 MiB buffer written before every timed step"},
        "voxels_per_s": world * sum(int(np.prod(a.shape)) for a in imgs) / (ms / 1e3),
        "total_walker_steps": steps, "sweeps": rep.get("sweeps"), "sort_edge": rep.get("sort_edge"),
        "sweep_steps": rep.get("sweep_steps"),
        "e2e": {"value": world * steps / e2e_s, "unit": "walker-steps/s", "seconds": e2e_s,
                "h2d_bytes_per_step": int(sum(a.nbytes for a in imgs) + sum(a.nbytes for a in labs)),
                "d2h_bytes_per_step": int(sum(v.nbytes for r in out if r for v in r.values()))},
        "clocks": clocks.summary(),
    }
    if rank == 0:
        print(json.dumps(line))


def launches_since(before, sweeps=0):
    """Kernel launches of libsmartinterp calls made since the `before`
    snapshot of _native.CALLS (si_walk_sorted: 6 per sweep + 4)."""
    from biomedisa_gb300 import _native as nat

    n = 0
    for k, v in nat.CALLS.items():
        d = v - before.get(k, 0)
        if k == "si_walk_sorted":
            n += 6 * sweeps + 4 * d
        else:
            n += MULTI_LAUNCH.get(k, 1) * d
    return n


def peaks():
    pk = ROOT / "MEASURED_PEAKS.json"
    return json.loads(pk.read_text()) if pk.exists() else {}


def surrogate_samples(count=16, shape=(128, 128, 128)):
    from biomedisa_gb300 import surrogate as SG

    return SG.training_set(count, shape=shape, mix=0.5, seed=7)


def trained_surrogate():
    """The hybrid's network: trained here (128 walked 96^3 volumes, 70 %
    large-style, 5000 AdamW steps on batches of 4 windows) or read back from the
    bench cache directory."""
    import torch

    from biomedisa_gb300 import surrogate as SG

    cache = Path(os.environ.get("SI_BENCH_CACHE", "/tmp")) / "si_surrogate_c16_d1248_n128_s5000_v2.pt"
    if cache.exists():
        return SG.load(cache), {"trained": False, "cache": str(cache)}
    t0 = time.perf_counter()
    net = SG.SurrogateNet(seed=0)
    samples = SG.training_set(128, mix=0.7, seed=0)
    t1 = time.perf_counter()
    losses = SG.train(net, samples, 5000, seed=0)
    torch.cuda.synchronize()
    info = {"trained": True, "samples_s": t1 - t0, "train_s": time.perf_counter() - t1,
            "loss_first100": float(np.mean(losses[:100])), "loss_last100": float(np.mean(losses[-100:]))}
    try:
        SG.save(net, cache)
    except OSError:
        pass
    return net, info


def nn_cpu_baseline(net, target_seconds=10.0):
    """The float64 NumPy oracle's forward + backward of the same network on
    one 32^3 window, repeated for about target_seconds (1 core)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import nn_oracle as NO

    rng = np.random.default_rng(0)
    n = 32
    x = NO.bf16_round(rng.uniform(0, 1, (1, n, n, n, 16)))
    ws = [c.w.cpu().numpy().astype(np.float64) for c in net.convs]
    bs = [c.b.cpu().numpy().astype(np.float64) for c in net.convs]
    p = rng.dirichlet(np.ones(4), size=(1, n, n, n))
    w = np.ones((1, n, n, n))
    t0, reps = time.perf_counter(), 0
    while True:
        NO.network_grads(x, ws, bs, list(net.dilations), p, w, 4)
        reps += 1
        if time.perf_counter() - t0 >= target_seconds:
            break
    secs = time.perf_counter() - t0
    return {"value": reps * n ** 3 / secs, "unit": "voxels/s", "cores": 1, "kind": "port",
            "sample": f"{reps} forward+backward passes of one 32^3 window through the float64 NumPy oracle "
                      f"(oracle/nn_oracle.py network_grads), {secs:.1f} s"}


def conv_cpu_baseline(c, target_seconds=10.0):
    """The float64 NumPy oracle's 16->16 convolution (bias, residual, ReLU)
    of the same layer on a (1, 16, 32, 128) window, repeated for about
    target_seconds (1 core)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import nn_oracle as NO

    rng = np.random.default_rng(0)
    shape = (1, 16, 32, 128)
    x = NO.bf16_round(rng.standard_normal(shape + (16,)) * 0.5)
    res = NO.bf16_round(rng.standard_normal(shape + (16,)) * 0.5)
    w = c.w.cpu().numpy().astype(np.float64)
    b = c.b.cpu().numpy().astype(np.float64)
    vox = int(np.prod(shape))
    t0, reps = time.perf_counter(), 0
    while True:
        np.maximum(NO.conv_fwd(x, w, b, c.dil) + res, 0)
        reps += 1
        if time.perf_counter() - t0 >= target_seconds:
            break
    secs = time.perf_counter() - t0
    return {"value": reps * vox / secs, "unit": "voxels/s", "cores": 1, "kind": "port",
            "sample": f"{reps} convolutions of a (1,16,32,128) window through the float64 NumPy oracle "
                      f"(oracle/nn_oracle.py conv_fwd + residual + ReLU), {secs:.1f} s"}


def run_train_bench(args, wl):
    """Surrogate training throughput: one step = forward, backward and AdamW
    over a batch of 8 windows of 64^3 (device-resident training set)."""
    import torch

    from biomedisa_gb300 import _native as nat
    from biomedisa_gb300 import surrogate as SG

    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned surrogate; nothing "
                              "to train"}))
        return
    world, rank, local = dist_setup()
    samples = surrogate_samples()
    net = SG.SurrogateNet(seed=0)
    batch, patch = 8, 64
    for i in range(args.warmup):
        SG.train(net, samples, 1, batch=batch, patch=patch, seed=100 + i)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    l2buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    times, launches = [], 0
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            flush_l2(l2buf)
            torch.cuda.synchronize()
            barrier(world)
            before = dict(nat.CALLS)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            SG.train(net, samples, 1, batch=batch, patch=patch, seed=200 + i)
            e.record(stream)
            torch.cuda.synchronize()
            barrier(world)
            times.append(s.elapsed_time(e))
            launches = launches_since(before)
    ms = max_over_ranks(world, sum(times) / len(times))
    vox = batch * patch ** 3
    value = world * vox / (ms / 1e3)
    # conv roofline: every conv runs forward, data gradient (except the stem) and weight gradient
    flops = 0
    for k, c in enumerate(net.convs):
        per = 2 * 27 * c.cin * c.cout * vox
        flops += per * (3 if k > 0 else 2)
    # per-kernel CUDA-event timing of the 16->16 forward convolution on one batch
    x = torch.randn((batch, patch, patch, patch, 16), device="cuda").to(torch.bfloat16)
    c = net.convs[1]
    shape = (batch, patch, patch, patch)
    for _ in range(3):
        SG.conv_fwd(x, c, shape, relu=True, tensor_core=net.tensor_core)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for _ in range(20):
        SG.conv_fwd(x, c, shape, relu=True, tensor_core=net.tensor_core)
    e.record(stream)
    torch.cuda.synchronize()
    conv_ms = s.elapsed_time(e) / 20
    conv_tflops = 2 * 27 * 16 * 16 * vox / (conv_ms / 1e3) / 1e12
    pk = peaks()
    bf16 = float(pk.get("bf16_tflops", 1900.0))
    kind = "measured" if "bf16_tflops" in pk else "fallback"
    e2e_t = []
    for i in range(args.e2e_steps or args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        SG.train(net, samples, 1, batch=batch, patch=patch, seed=300 + i)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(world, sum(e2e_t) / len(e2e_t))
    line = {
        "metric": "training voxels/s", "value": value, "unit": "voxels/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16", "data": "synthetic (walked procedural volumes; targets = hit fractions of the walk)",
        "config": {"workload": wl["desc"], "global_batch": batch, "seq_len": patch ** 3,
                   "parallelism": "single GPU", "l2": "256 MiB buffer written before every timed step"},
        "step_tflops": flops / (ms / 1e3) / 1e12,
        "e2e": {"value": world * vox / e2e_s, "unit": "voxels/s", "seconds": e2e_s, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 4,
                "note": "the public training call (surrogate.train) on the device-resident training set; the loss "
                        "(4 bytes) is read back each step"},
        "gpu_launches": launches,
        "roofline": {"bound": "tensor", "achieved": conv_tflops, "peak": bf16, "unit": "TFLOP/s",
                     "frac": conv_tflops / bf16, "traffic": None,
                     "note": f"16->16 forward convolution ({'conv16_umma_kernel, tcgen05' if net.tensor_core else 'conv16_kernel, mma.sync'} "
                             f"bf16), 2*27*16*16 FLOP per output voxel x {vox} voxels / CUDA-event time; peak "
                             f"{kind} bf16 (cuBLAS burst)"},
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = nn_cpu_baseline(net, min(args.ref_seconds, 20.0))
    if rank == 0:
        print(json.dumps(line))


def run_conv16_bench(args, wl):
    """The surrogate's 16->16 convolution alone: one step = one forward
    convolution on the tensor cores (si_nn_conv16_tc) of a (1,128,256,1024)
    bf16 volume with bias, residual and ReLU; the mma.sync kernel is timed on
    the same input beside it, and ``e2e`` runs the same call on pinned host
    arrays (input and residual in, output out)."""
    import torch

    from biomedisa_gb300 import _native as nat
    from biomedisa_gb300 import surrogate as SG

    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned surrogate and no "
                              "convolution"}))
        return
    world, rank, local = dist_setup()
    shape = (1, 128, 256, 1024)
    vox = shape[0] * shape[1] * shape[2] * shape[3]
    net = SG.SurrogateNet(seed=0)
    c = net.convs[1]
    gen = torch.Generator(device="cuda").manual_seed(7)
    x = (torch.randn(shape + (16,), device="cuda", generator=gen) * 0.5).to(torch.bfloat16)
    res = (torch.randn(shape + (16,), device="cuda", generator=gen) * 0.5).to(torch.bfloat16)

    def conv(xi, ri, tc=True):
        return SG.conv_fwd(xi, c, shape, relu=True, residual=ri, tensor_core=tc)

    for _ in range(args.warmup):
        conv(x, res)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    l2buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    times, launches = [], 0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush_l2(l2buf)
            torch.cuda.synchronize()
            barrier(world)
            before = dict(nat.CALLS)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            y = conv(x, res)
            e.record(stream)
            torch.cuda.synchronize()
            barrier(world)
            times.append(s.elapsed_time(e))
            launches = launches_since(before)
    SG.umma_check()
    ms = max_over_ranks(world, sum(times) / len(times))
    flops = 2 * 27 * 16 * 16 * vox
    tflops = flops / (ms / 1e3) / 1e12
    mma_t = []
    for _ in range(max(3, args.steps)):
        flush_l2(l2buf)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        ym = conv(x, res, tc=False)
        e.record(stream)
        torch.cuda.synchronize()
        mma_t.append(s.elapsed_time(e))
    mma_ms = sum(mma_t) / len(mma_t)
    diff = float((ym.float() - y.float()).abs().max())
    xh, rh = x.cpu().pin_memory(), res.cpu().pin_memory()
    yh = torch.empty(shape + (16,), dtype=torch.bfloat16).pin_memory()
    e2e_t = []
    for _ in range(args.e2e_steps or args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        yd = conv(xh.to("cuda", non_blocking=True), rh.to("cuda", non_blocking=True))
        yh.copy_(yd, non_blocking=True)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    SG.umma_check()
    e2e_s = max_over_ranks(world, sum(e2e_t) / len(e2e_t))
    act = vox * 16 * 2
    pk = peaks()
    bf16 = float(pk.get("bf16_tflops", 1900.0))
    kind = "measured" if "bf16_tflops" in pk else "fallback"
    hbm = float(pk.get("hbm_gbs", 6800.0))
    line = {
        "metric": "voxels/s", "value": world * vox / (ms / 1e3), "unit": "voxels/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16", "data": "synthetic (seeded normal activations, the network's own "
        "initial weights)",
        "config": {"workload": wl["desc"], "global_batch": 1, "parallelism": "single GPU",
                   "l2": "256 MiB buffer written before every timed step; activations 1 GiB > L2"},
        "mma_sync_ms": mma_ms, "speedup_vs_mma_sync": mma_ms / ms, "max_abs_diff_vs_mma_sync": diff,
        "e2e": {"value": world * vox / e2e_s, "unit": "voxels/s", "seconds": e2e_s, "h2d_bytes_per_step": 2 * act,
                "d2h_bytes_per_step": act,
                "note": "the same call on pinned host arrays: input and residual copied in, output copied out"},
        "gpu_launches": launches,
        "roofline": {"bound": "tensor", "achieved": tflops, "peak": bf16, "unit": "TFLOP/s", "frac": tflops / bf16,
                     "traffic": None,
                     "hbm_frac": 3 * act / (ms / 1e3) / 1e9 / hbm,
                     "note": f"conv16_umma_kernel: 2*27*16*16 FLOP per output voxel x {vox} voxels / CUDA-event "
                             f"time; peak {kind} bf16 (cuBLAS burst); hbm_frac = (input + residual + output, "
                             f"96 B per voxel) / time over the {kind} HBM copy bandwidth"},
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = conv_cpu_baseline(c, min(args.ref_seconds, 10.0))
    if rank == 0:
        print(json.dumps(line))


def run_hybrid_bench(args, wl):
    """Hybrid (surrogate + restricted walk) vs the plain job on the large
    volume; value = voxels/s of the hybrid on device-resident inputs."""
    import torch

    from biomedisa_gb300 import _native as nat
    from biomedisa_gb300 import interpolation as I
    from biomedisa_gb300 import surrogate as SG

    if args.impl == "reference":
        world = int(os.environ.get("WORLD_SIZE", "1"))
        if int(os.environ.get("RANK", "0")) != 0:
            return
        img, lab = make_inputs("large")
        cb = cpu_baseline(img, lab, wl, args.ref_seconds)
        line = {"metric": "voxels/s", "unit": "voxels/s", "impl": "reference"}
        # the reference walks every seed: extrapolate its walker rate to the whole plain walk
        seeds_total = reference_seed_count(lab)
        secs = seeds_total * wl["nbrw"] * wl["sorw"] / cb["value"]
        v = int(np.prod(img.shape)) / secs
        line.update(value=v, n_gpus=world, steps=args.steps, warmup=args.warmup, ms_per_step=secs * 1e3,
                    higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32", data="synthetic",
                    config={"workload": wl["desc"], "global_batch": 1, "parallelism": "host cores"},
                    cpu_baseline={"value": v, "unit": "voxels/s", "cores": cb["cores"], "kind": cb["kind"],
                                  "sample": cb["sample"] + f"; extrapolated to all {seeds_total} seeds"},
                    e2e={"value": v, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
        print(json.dumps(line))
        return
    world, rank, local = dist_setup()
    img, lab = make_inputs("large")
    net, train_info = trained_surrogate()
    data, labels = I.normalize_host_dtypes(img, lab)
    icode, lcode = I._IMG_DTYPES[data.dtype], I._LAB_DTYPES[labels.dtype]
    img_t, lab_t = I.upload(data, labels)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    # the yardstick: one plain job (same entry points as the large workload, smooth=0)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record(stream)
    job, res = run_job(img_t, icode, lab_t, lcode, wl)
    ev[1].record(stream)
    torch.cuda.synchronize()
    plain_ms = ev[0].elapsed_time(ev[1])
    plain = res["regular"]
    plain_smooth = res.get("smooth")
    plain_steps = job.total_steps()
    present = sorted(int(v) for v in np.unique(lab[::12]))
    del job, res
    torch.cuda.empty_cache()
    kw = dict(threshold=wl["threshold"], radius=wl["radius"], coarse=wl["coarse"], grow=wl["grow"],
              nbrw=wl["nbrw"], sorw=wl["sorw"], smooth=wl["smooth"])
    for _ in range(args.warmup):
        r, _ = SG.hybrid_interpolation(None, None, net, device_inputs=(img_t, icode, lab_t, lcode), **kw)
        del r
    torch.cuda.synchronize()
    l2buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    times, launches, st, dice, dice_smooth = [], 0, {}, {}, {}
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush_l2(l2buf)
            torch.cuda.synchronize()
            barrier(world)
            before = dict(nat.CALLS)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            r, st = SG.hybrid_interpolation(None, None, net, device_inputs=(img_t, icode, lab_t, lcode), **kw)
            e.record(stream)
            torch.cuda.synchronize()
            barrier(world)
            times.append(s.elapsed_time(e))
            launches = launches_since(before, st["sweeps"])
            dice = SG.label_dice(r["regular"], plain, present)
            dice_smooth = SG.label_dice(r["smooth"], plain_smooth, present) if plain_smooth is not None else {}
            del r
    ms = max_over_ranks(world, sum(times) / len(times))
    vox = int(np.prod(img.shape))
    # end to end: host arrays in, host labels out
    t_e2e = []
    out_bytes = 0
    for _ in range(args.e2e_steps or args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r, _ = SG.hybrid_interpolation(img, lab, net, **kw)
        out = r["regular"].cpu().numpy()
        t_e2e.append(time.perf_counter() - t0)
        out_bytes = out.nbytes
        del r
    e2e_s = max_over_ranks(world, sum(t_e2e) / len(t_e2e))
    pk = peaks()
    hbm = float(pk.get("hbm_gbs", 6800.0))
    kind = "measured" if "hbm_gbs" in pk else "fallback"
    walk_rate = st["walker_steps"] / (st["walk_ms_events"] / 1e3) if st.get("walk_ms_events") else None
    achieved = walk_rate * WALK_BYTES_PAYLOAD_U8 / 1e9 if walk_rate else None
    line = {
        "metric": "voxels/s", "value": world * vox / (ms / 1e3), "unit": "voxels/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded generator, no public dataset)",
        "config": {"workload": wl["desc"], "global_batch": 1, "parallelism": "single GPU",
                   "l2": "256 MiB buffer written before every timed step; hit maps 30 GB > L2"},
        "plain_ms": plain_ms, "plain_voxels_per_s": vox / (plain_ms / 1e3), "speedup_vs_plain": plain_ms / ms,
        "dice_vs_plain": {str(k): round(v, 5) for k, v in dice.items()},
        "dice_min": min(dice.values()) if dice else None,
        "dice_smooth_vs_plain": {str(k): round(v, 5) for k, v in dice_smooth.items()},
        "dice_smooth_min": min(dice_smooth.values()) if dice_smooth else None,
        "threshold": wl["threshold"],
        "frac_uncertain": st.get("frac_uncertain"), "frac_seeds_walked": st.get("frac_seeds_walked"),
        "walker_steps": st.get("walker_steps"), "plain_walker_steps": plain_steps,
        "seconds_surrogate": st.get("seconds_surrogate"), "seconds_walk": st.get("seconds_walk"),
        "surrogate": train_info,
        "e2e": {"value": world * vox / e2e_s, "unit": "voxels/s", "seconds": e2e_s,
                "h2d_bytes_per_step": int(img.nbytes + lab.nbytes), "d2h_bytes_per_step": int(out_bytes)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm if achieved else None, "traffic": None,
                     "note": f"restricted walk (sweep_kernel): {WALK_BYTES_PAYLOAD_U8} B/step logical payload x "
                             f"steps / CUDA-event walk time; peak {kind} (hbm_gbs)"},
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cb = cpu_baseline(img, lab, wl, args.ref_seconds)
            secs = plain_steps / cb["value"]
            line["cpu_baseline"] = {"value": vox / secs, "unit": "voxels/s", "cores": cb["cores"],
                                    "kind": cb["kind"],
                                    "sample": cb["sample"] + f"; extrapolated to the plain walk's {plain_steps} "
                                                             "steps"}
        except Exception as ex:
            line["cpu_baseline"] = {"value": None, "unit": "voxels/s", "cores": 0, "kind": "reference",
                                    "sample": f"unavailable: {ex}"}
    if rank == 0:
        print(json.dumps(line))


def acwe_inputs():
    """The active-contour workload: image and jittered segmentation of three
    ellipsoids (biomedisa_gb300.synthetic.blob_volume)."""
    from biomedisa_gb300.synthetic import blob_volume

    cache = Path(os.environ.get("SI_BENCH_CACHE", "/tmp")) / "si_bench_acwe_0.npz"
    if cache.exists():
        z = np.load(cache)
        return z["img"], z["lab"]
    img, lab = blob_volume((256, 384, 384), 11, [1, 2, 3], [(128, 192, 192), (90, 120, 250), (170, 260, 130)],
                           [(90, 120, 130), (40, 50, 45), (50, 40, 45)], 14.0, jitter=6.0)
    lab = lab.astype(np.uint8)
    try:
        np.savez(cache, img=img, lab=lab)
    except OSError:
        pass
    return img, lab


def acwe_cpu_sample(img, lab):
    """Bounded sample for the CPU leg: a 48 x 96 x 96 block across the border
    of the largest ellipsoid."""
    sl = (slice(104, 152), slice(24, 120), slice(150, 246))
    return np.ascontiguousarray(img[sl]), np.ascontiguousarray(lab[sl])


def time_acwe_oracle(img, lab, wl, reps):
    sys.path.insert(0, str(ROOT / "oracle"))
    import acwe_oracle as A

    si, sl = acwe_cpu_sample(img, lab)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        A.active_contour(si, sl, 1.0, 1, 3)
        A.active_contour(si, sl, simple=True)
        times.append(time.perf_counter() - t0)
    secs = statistics.median(times)
    return {"value": si.size / secs, "unit": "voxels/s", "cores": 1, "kind": "port",
            "sample": f"a {si.shape[0]}x{si.shape[1]}x{si.shape[2]} block across an object border, both modes; the "
                      "reference's numba activeContour restated in NumPy (oracle/acwe_oracle.py; numba is not "
                      "installed), one process"}


def run_acwe_bench(args, wl):
    """Active contour: value = volume voxels / (both activeContour modes) on
    device-resident inputs; e2e through activeContour with numpy in/out;
    roofline of the refinement's chamfer band."""
    import torch

    from biomedisa_gb300 import _native as nat
    from biomedisa_gb300 import active_contour as AC
    from biomedisa_gb300 import interpolation as I

    world = int(os.environ.get("WORLD_SIZE", "1"))
    if int(os.environ.get("RANK", "0")) != 0:  # one GPU's job; other ranks exit without work
        return
    img, lab = acwe_inputs()
    n_vox = int(np.prod(img.shape))
    if args.impl == "reference":
        cb = time_acwe_oracle(img, lab, wl, max(args.steps, 1))
        print(json.dumps({
            "metric": "voxels/s", "value": cb["value"], "unit": "voxels/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": n_vox / cb["value"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8/f32/f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": wl["desc"], "global_batch": 1, "parallelism": "host cores"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    img_t, lab_t = I.upload(img, lab)
    Z, Y, X = img.shape
    l2buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def run(scan_events=None):
        frame = AC.Frame(img_t, nat.SI_U8, (1, 1, 1), (Z, Y, X))
        all_labels = AC.label_list(lab_t)
        r = AC.AcweRun(frame, lab_t, all_labels)
        r.gather()
        a = r.acwe(1.0, 1, 3)
        f = r.refined(scan_events)
        return r, a, f

    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    t_job, t_scan, launches = [], [], 0
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            flush_l2(l2buf)
            torch.cuda.synchronize()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            ev[0].record(stream)
            r, _, _ = run((ev[2], ev[3]))
            ev[1].record(stream)
            torch.cuda.synchronize()
            t_job.append(ev[0].elapsed_time(ev[1]))
            t_scan.append(ev[2].elapsed_time(ev[3]))
            launches += r.launches
    ms = sum(t_job) / len(t_job)
    scan_ms = sum(t_scan) / len(t_scan)
    z0, y0, x0, cZ, cY, cX = r.box
    AC.activeContour(img, lab, 1.0, 1, 3)
    t_e2e, out_bytes = [], 0
    for _ in range(args.steps):
        flush_l2(l2buf)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        o1 = AC.activeContour(img, lab, 1.0, 1, 3)
        o2 = AC.activeContour(img, lab, simple=True)
        t_e2e.append(time.perf_counter() - t0)
        out_bytes = o1.nbytes + o2.nbytes
    e2e_s = sum(t_e2e) / len(t_e2e)
    # the chamfer band: 10 Jacobi passes, each reading and writing the float32
    # distance of every crop voxel
    bytes_alg = 10 * 8 * cZ * cY * cX
    achieved = bytes_alg / (scan_ms / 1e3) / 1e9
    hbm = float(peaks().get("hbm_gbs", 6800.0))
    line = {
        "metric": "voxels/s", "value": n_vox / (ms / 1e3), "unit": "voxels/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8/f32", "data": "synthetic (seeded generator, no public dataset)",
        "config": {"workload": wl["desc"], "global_batch": 1, "parallelism": "single GPU",
                   "l2": "256 MiB buffer written before every timed step", "crop": [cZ, cY, cX]},
        "e2e": {"value": n_vox / e2e_s, "unit": "voxels/s", "seconds": e2e_s,
                "h2d_bytes_per_step": 2 * int(img.nbytes + lab.nbytes), "d2h_bytes_per_step": int(out_bytes)},
        "gpu_launches": launches // max(args.steps, 1),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None, "kernel_ms": scan_ms,
                     "note": "the refinement's chamfer band (si_acwe_chamfer_band: 10 Jacobi passes of a "
                             "27-point min-plus stencil over the crop, each reading and writing 4 B per voxel) / "
                             "its CUDA-event time"},
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = time_acwe_oracle(img, lab, wl, 3)
    print(json.dumps(line))


def run_geodesic_bench(args, wl):
    """Geodesic interpolation: value = volume voxels / geodesic_segment time
    on device-resident inputs; e2e through geodesic_segment with numpy in/out;
    roofline of the wavefront kernel over the whole scan."""
    import torch

    from biomedisa_gb300 import geodis as D
    from biomedisa_gb300 import interpolation as I

    sys.path.insert(0, str(ROOT / "oracle"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:  # one GPU's job; the other ranks of a multi-GPU launch exit without work
        return
    img, lab = make_inputs("geodesic")
    n_vox = int(np.prod(img.shape))
    nol = len(np.unique(lab[lab >= 0]))
    if args.impl == "reference":
        import geo_oracle as G

        times = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            G.geodesic_segment(img, lab)
            if i >= args.warmup:
                times.append(time.perf_counter() - t0)
        secs = statistics.median(times)
        v = n_vox / secs
        print(json.dumps({
            "metric": "voxels/s", "value": v, "unit": "voxels/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": secs * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": wl["desc"], "global_batch": 1, "parallelism": "host cores"},
            "cpu_baseline": {"value": v, "unit": "voxels/s", "cores": 1, "kind": "port",
                             "sample": "the whole volume; the reference's numba scan restated in C "
                                       "(oracle/geo_oracle.c; numba is not installed), one core"},
            "e2e": {"value": v, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    img_t, lab_t = I.upload(img, lab)
    code_i, code_l = I._IMG_DTYPES[img.dtype], I._LAB_DTYPES[lab.dtype]
    l2buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        D.geodesic_segment_device(img_t, code_i, lab_t, code_l)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    t_job, t_scan = [], []
    # the scan alone, for the wavefront kernel's roofline (same inputs as a job)
    work = torch.empty(img.shape, dtype=torch.float32, device="cuda")
    mm = torch.empty(4, dtype=torch.int32, device="cuda")
    from biomedisa_gb300 import _native as nat

    nat.call("si_geo_normalize", img_t.data_ptr(), code_i, n_vox, work.data_ptr(), mm.data_ptr(),
             stream.cuda_stream)
    c0 = torch.full((nol,) + img.shape, float("inf"), dtype=torch.float32, device="cuda")
    c0[:, ::9, ::11, ::13] = 0.0
    scan_ms_mode = {}
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            flush_l2(l2buf)
            torch.cuda.synchronize()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record(stream)
            D.geodesic_segment_device(img_t, code_i, lab_t, code_l)
            ev[1].record(stream)
            torch.cuda.synchronize()
            t_job.append(ev[0].elapsed_time(ev[1]))
        cbuf = torch.empty_like(c0)  # one buffer: auto mode keys its graph by the pointers
        for mode in range(6):
            for _ in range(2):  # untimed: auto mode captures its graph on the second call
                cbuf.copy_(c0)
                D.scan_device(cbuf, work, mode=mode)
            t_scan = []
            for _ in range(args.steps):
                cbuf.copy_(c0)
                c = cbuf
                flush_l2(l2buf)
                torch.cuda.synchronize()
                ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                ev[0].record(stream)
                D.scan_device(c, work, mode=mode)
                ev[1].record(stream)
                torch.cuda.synchronize()
                t_scan.append(ev[0].elapsed_time(ev[1]))
            scan_ms_mode[mode] = sum(t_scan) / len(t_scan)
    ms = sum(t_job) / len(t_job)
    scan_ms = scan_ms_mode[D.SCAN_AUTO]
    D.geodesic_segment(img, lab)
    t_e2e = []
    for _ in range(args.steps):
        flush_l2(l2buf)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = D.geodesic_segment(img, lab)
        t_e2e.append(time.perf_counter() - t0)
    e2e_s = sum(t_e2e) / len(t_e2e)
    scan_launches = D.scan_launches(img.shape)
    waves = D.scan_launches(img.shape, mode=D.SCAN_WAVEFRONTS)
    Z, Y, X = img.shape
    updates = 4 * ((Z - 1) * (Y - 2) * (X - 2)) * 2 * nol  # voxel-label updates of one scan
    bytes_alg = updates * (8 + 4 / nol)  # read + write the distance, the image shared by the labels
    achieved = bytes_alg / (scan_ms / 1e3) / 1e9
    pk = peaks()
    hbm = float(pk.get("hbm_gbs", 6800.0))
    line = {
        "metric": "voxels/s", "value": n_vox / (ms / 1e3), "unit": "voxels/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded generator, no public dataset)",
        "config": {"workload": wl["desc"], "global_batch": 1, "parallelism": "single GPU",
                   "l2": "256 MiB buffer written before every timed step"},
        "e2e": {"value": n_vox / e2e_s, "unit": "voxels/s", "seconds": e2e_s,
                "h2d_bytes_per_step": int(img.nbytes + lab.nbytes), "d2h_bytes_per_step": int(r.nbytes)},
        "gpu_launches": 3 + 1 + 1 + scan_launches + 1,
        "scan_ms": scan_ms, "scan_mode": "tiles in skewed coordinates, launches replayed from a cached CUDA graph",
        "scan_ms_by_mode": {"tiles": scan_ms_mode[D.SCAN_TILES], "tiles_graph": scan_ms_mode[D.SCAN_TILE_GRAPH],
                            "wavefronts": scan_ms_mode[D.SCAN_WAVEFRONTS],
                            "wavefronts_graph": scan_ms_mode[D.SCAN_WAVEFRONT_GRAPH],
                            "cluster": scan_ms_mode[D.SCAN_CLUSTER]},
        "wavefronts_per_scan": waves, "launches_per_scan": scan_launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None,
                     "note": f"geo_tile_kernel over one scan ({scan_launches} launches of tile-wavefronts, "
                             f"{nol} labels): algorithmic bytes = 8 B per voxel-label update (read + write the "
                             "distance) + 4 B per voxel update (image) / CUDA-event scan duration; latency-bound: "
                             "the tile-wavefronts run one after another, each tile steps through its 32 planes; "
                             f"peak {'measured' if pk else 'fallback'} HBM"},
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        import geo_oracle as G

        t0 = time.perf_counter()
        G.geodesic_segment(img, lab)
        secs = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n_vox / secs, "unit": "voxels/s", "cores": 1, "kind": "port",
                                "sample": "the whole volume; the reference's numba scan restated in C "
                                          "(oracle/geo_oracle.c), one core"}
    print(json.dumps(line))


def profile_jobs(args, wl):
    """Untimed jobs on device-resident inputs, for profiler captures."""
    import torch

    from biomedisa_gb300 import interpolation as I

    torch.cuda.set_device(0)
    if args.host_loop:
        from biomedisa_gb300 import _native as nat

        nat.call("si_walk_sorted_set_loop", 0)
    img, lab = make_inputs(args.workload)
    data, labels = I.normalize_host_dtypes(img, lab)
    img_t, lab_t = I.upload(data, labels)
    for _ in range(args.profile_jobs):
        t0 = time.perf_counter()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        job, _ = run_job(img_t, I._IMG_DTYPES[data.dtype], lab_t, I._LAB_DTYPES[labels.dtype], wl, events=ev)
        torch.cuda.synchronize()
        walk_s = ev[0].elapsed_time(ev[1]) / 1e3
        print(f"job: {job.total_steps()} walker steps, {time.perf_counter() - t0:.3f} s, walk {walk_s:.3f} s "
              f"({job.total_steps() / walk_s:.3e} steps/s), walker={job.walker_used}, "
              f"sweeps={getattr(job, 'rounds', None)}, crop={job.cplan.crop}, seeds={int(job.n_seeds.item())}",
              flush=True)


def measure_l2(torch):
    """L2 ceilings measured here with the library's probe kernels: read
    bandwidth over a 48 MiB L2-resident buffer (L1 bypassed, best of 10) and
    random 4-byte atomic adds into a 16 MiB buffer (one 32-byte sector each)."""
    from biomedisa_gb300 import _native as nat

    stream = torch.cuda.current_stream().cuda_stream
    buf = torch.zeros(48 << 20, dtype=torch.uint8, device="cuda")
    sink = torch.zeros(1, dtype=torch.int32, device="cuda")
    reps = 20
    nat.call("si_probe_l2_read", buf.data_ptr(), buf.numel(), 2, sink.data_ptr(), stream)
    best_read = 0.0
    for _ in range(10):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        nat.call("si_probe_l2_read", buf.data_ptr(), buf.numel(), reps, sink.data_ptr(), stream)
        e.record()
        torch.cuda.synchronize()
        best_read = max(best_read, reps * buf.numel() / (s.elapsed_time(e) / 1e3) / 1e9)
    words = 1 << 22
    abuf = torch.zeros(words, dtype=torch.int32, device="cuda")
    n = 1 << 30
    nat.call("si_probe_l2_atomics", abuf.data_ptr(), words, 1 << 24, stream)
    best_atom = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        nat.call("si_probe_l2_atomics", abuf.data_ptr(), words, n, stream)
        e.record()
        torch.cuda.synchronize()
        best_atom = max(best_atom, n / (s.elapsed_time(e) / 1e3))
    return {"read_gbs": best_read, "atomics_per_s": best_atom}


if __name__ == "__main__":
    main()
