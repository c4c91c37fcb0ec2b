"""The allocation-free seed extraction entry point (si_extract_seeds_noalloc).

It exists for callers that cannot allocate device memory while extracting
seeds — a plug-in whose host application owns the GPU's memory pool, or a
pipeline that must avoid cudaMalloc's device-wide synchronisation — and keeps
its per-row counters in a fixed device array of the library instead. The test
calls it through the C ABI twice in a row, on two different volumes, and
requires the same seeds and seed count as si_extract_seeds with a caller
buffer (integer/bit-pattern data: exact equality is the tolerance)."""
import numpy as np
import pytest
import torch

from biomedisa_gb300 import _native as nat
from biomedisa_gb300 import interpolation as I
from biomedisa_gb300.synthetic import plain_volume, sparse_labels

pytestmark = pytest.mark.gpu


def _prepared(img, lab, allaxis):
    d, l = I.normalize_host_dtypes(img, lab)
    ti, tl = I.upload(d, l)
    job = I.DeviceJob(ti, I._IMG_DTYPES[d.dtype], tl, I._LAB_DTYPES[l.dtype], allaxis=allaxis)
    assert job.analyze() is None
    job.prepare()  # runs si_extract_seeds with a caller-provided counter buffer
    torch.cuda.synchronize()
    return job


def _noalloc_seeds(job):
    cp, dev = job.cplan, job.dev
    n_sl = len(cp.slice_list)
    sl = torch.from_numpy(np.ascontiguousarray(cp.slice_list.reshape(-1))).to(dev)
    slot_lut = torch.from_numpy(job.lplan.slot_lut).to(dev)
    seeds = torch.full_like(job.seeds, 0xAB)
    n_seeds = torch.full((1,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    nat.call("si_extract_seeds_noalloc", job.lab.data_ptr(), job.lab_code, *job.shape0, *cp.crop,
             slot_lut.data_ptr(), job.slot_label.data_ptr(), job.work.data_ptr(), int(job.work_is_float),
             sl.data_ptr(), n_sl, seeds.data_ptr(), n_seeds.data_ptr(), stream)
    torch.cuda.synchronize()
    return seeds, int(n_seeds.item())


def test_noalloc_seed_extraction_matches_two_calls_in_a_row(cuda):
    img_a, _, truth_a = plain_volume(seed=31, shape=(40, 44, 42), z_every=5, semi=(7, 13))
    lab_a = sparse_labels(truth_a.astype(np.int32), z_every=5, y_every=7, x_every=6)
    img_b, lab_b, _ = plain_volume(seed=32, shape=(30, 26, 34), z_every=3, semi=(5, 10))
    for img, lab, allaxis in ((img_a, lab_a, True), (img_b, lab_b, False)):
        job = _prepared(img, lab, allaxis)
        n_ref = int(job.n_seeds.item())
        assert n_ref > 0
        seeds, n = _noalloc_seeds(job)
        assert n == n_ref
        assert torch.equal(seeds[: 16 * n], job.seeds[: 16 * n])


def test_noalloc_rejects_sizes_beyond_its_static_scratch(cuda):
    lib = nat.lib()
    # 2000 slices x 1000 rows needs 2,000,001 counters > 1,048,576: rejected before any launch
    dummy = torch.zeros(16, dtype=torch.int32, device=cuda)
    p = dummy.data_ptr()
    rc = lib.si_extract_seeds_noalloc(p, nat.SI_I32, 10, 10, 10, 0, 0, 0, 1000, 1000, 10, p, p, p, 0, p, 2000, p, p,
                                      torch.cuda.current_stream().cuda_stream)
    assert rc == 3
    assert b"static scratch" in lib.si_last_error()
