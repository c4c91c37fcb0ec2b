"""Worker processes of tests/test_dist_cpu.py (gloo, CPU only)."""
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def _init(rank, world, port):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    return dist


def bench_timing(rank, world, port, out):
    """bench.py's barrier and max-over-ranks on gloo ranks."""
    sys.path.insert(0, str(ROOT))
    import bench

    dist = _init(rank, world, port)
    bench.barrier(world)
    v = bench.max_over_ranks(world, 10.0 + rank)
    np.save(out / f"timing_{rank}.npy", np.array([v]))
    dist.destroy_process_group()


def sharded_walk(rank, world, port, out):
    """Each rank walks its share of the seeds with the oracle; an integer
    SUM all-reduce of the hit maps gives the whole walk (the multi-GPU design:
    seeds are independent and hits are integer sums)."""
    import torch

    sys.path.insert(0, str(ROOT / "oracle"))
    sys.path.insert(0, str(ROOT))
    import oracle as O
    from biomedisa_gb300.synthetic import plain_volume

    dist = _init(rank, world, port)
    img, lab, _ = plain_volume(seed=21, shape=(22, 24, 26), z_every=4, semi=(4, 8))
    data = np.pad(O.normalize_image(img), 1)
    l2, all_labels = O.pre_processing(np.pad(lab, 1))
    idx, _ = O.read_labeled_slices(l2)
    seeds = O.extract_seeds(data, l2, [(0, k) for k in idx], all_labels)
    mine = O.subset_seeds(seeds, np.arange(len(seeds)) % world == rank)
    hits = O.walk_c(data, mine, 3, 50, 7, len(all_labels)).astype(np.int64)
    t = torch.from_numpy(hits)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    if rank == 0:
        np.save(out / "sharded.npy", t.numpy())
        np.save(out / "whole.npy", O.walk_c(data, seeds, 3, 50, 7, len(all_labels)).astype(np.int64))
    dist.barrier()
    dist.destroy_process_group()
