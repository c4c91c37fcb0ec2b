"""GPU parity of the curvature smoothing (si_smooth / si_smooth_f32) against
the oracle's restatement of the reference kernels (gpu_kernels.py:118-183),
bit for bit, in both update modes:
  * 'f32'     — phi + RN(0.01f * kappa) (binary32);
  * 'ref_f64' — the reference's own `phi += 0.01 * curvature`: binary64
                product with the binary64 literal 0.01 and binary64 sum,
                rounded to binary32 on the store (gpu_kernels.py:133).
Shapes cover row lengths that are not a multiple of 4 (pitched scratch),
volumes smaller than one CTA tile and larger than several, and sparse maps
whose support box is far smaller than the volume (CTAs outside it skip).
The last test makes the kernels' bounded waits run out and checks that the
status is reported and that the device stays usable."""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
from biomedisa_gb300 import _native as nat
from biomedisa_gb300 import smart_interpolation
from biomedisa_gb300.interpolation import SMOOTH_UPDATES, smooth_buffers, smooth_check
from biomedisa_gb300.synthetic import plain_volume

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (3, 3, 3), (5, 9, 66), (19, 23, 37), (40, 17, 130), (70, 20, 65)]


def _maps(shape, nol, sparse, seed):
    rng = np.random.default_rng(seed)
    m = (rng.random((nol,) + shape) * 50).astype(np.float32)
    if sparse:
        keep = np.zeros(shape, bool)
        z, y, x = shape
        keep[z // 3: z // 3 + max(1, z // 4), y // 2: y // 2 + max(1, y // 5), x // 4: x // 4 + max(1, x // 6)] = True
        m[:, ~keep] = 0.0
        m[-1] = 0.0  # an all-zero map: empty support box
    return m


def _run(maps_np, iters, update, hits):
    nol, Zc, Yc, Xc = maps_np.shape
    dev = torch.device("cuda")
    tmp0, tmp1 = smooth_buffers(Zc, Yc, Xc, dev)
    tmp1.fill_(123.0)  # the scratch holds another map's values: they must not leak into the result
    tmp0.fill_(-7.0)
    st = torch.cuda.current_stream().cuda_stream
    if hits:
        t = torch.from_numpy(maps_np.astype(np.uint32)).to(dev)
        nat.call("si_smooth", t.data_ptr(), tmp0.data_ptr(), tmp1.data_ptr(), nol, Zc, Yc, Xc, iters,
                 SMOOTH_UPDATES[update], st)
        smooth_check()
        return t.view(torch.float32).cpu().numpy()
    t = torch.from_numpy(maps_np).to(dev)
    nat.call("si_smooth_f32", t.data_ptr(), tmp0.data_ptr(), tmp1.data_ptr(), nol, Zc, Yc, Xc, iters,
             SMOOTH_UPDATES[update], st)
    smooth_check()
    return t.cpu().numpy()


@pytest.mark.parametrize("update", ["f32", "ref_f64"])
@pytest.mark.parametrize("shape", SHAPES, ids=[f"{z}x{y}x{x}" for z, y, x in SHAPES])
@pytest.mark.parametrize("sparse", [False, True], ids=["dense", "sparse"])
def test_float_maps_bit_exact(update, shape, sparse, cuda):
    maps = _maps(shape, 3, sparse, seed=sum(shape))
    for iters in (1, 2, 3, 6):
        got = _run(maps, iters, update, hits=False)
        exp = O.smooth(maps, iters, update)
        bad = np.count_nonzero(got.view(np.uint32) != exp.view(np.uint32))
        assert bad == 0, (update, shape, iters, bad)


@pytest.mark.parametrize("update", ["f32", "ref_f64"])
def test_hit_maps_bit_exact(update, cuda):
    hits = np.rint(_maps((21, 30, 45), 2, True, seed=4)).astype(np.float32)
    for iters in (0, 1, 5):
        got = _run(hits, iters, update, hits=True)
        exp = O.smooth(hits, iters, update) if iters else hits.astype(np.float32)
        bad = np.count_nonzero(got.view(np.uint32) != exp.view(np.uint32))
        assert bad == 0, (update, iters, bad)


def test_pipeline_reference_update_bit_exact(cuda):
    """smart_interpolation(smooth_update='ref_f64') reproduces the oracle in
    the reference's update arithmetic; the two modes agree on the regular
    labels and on almost every smoothed label."""
    img, lab, _ = plain_volume(seed=5, shape=(36, 40, 44), z_every=5, semi=(7, 13))
    kw = dict(nbrw=2, sorw=120)
    got = smart_interpolation(img, lab, smooth=20, smooth_update="ref_f64", rng_seed=11, **kw)
    exp = O.smart_interpolation(img, lab, smooth_iters=20, smooth_update="ref_f64", key=11, **kw)
    assert np.array_equal(got["smooth"], exp["smooth"]) and np.array_equal(got["regular"], exp["regular"])
    f32 = smart_interpolation(img, lab, smooth=20, rng_seed=11, **kw)
    assert np.array_equal(f32["regular"], got["regular"])
    assert np.mean(f32["smooth"] == got["smooth"]) > 0.99


@pytest.mark.parametrize("pairs", [1, 2])
@pytest.mark.parametrize("shape", [(9, 13, 70), (20, 17, 200), (6, 11, 129)], ids=["x70", "x200", "x129"])
def test_tile_widths_bit_exact(pairs, shape, cuda):
    """Both column widths of the smoothing kernel (64 and 128 voxels per CTA)
    give the oracle's maps, on rows that end inside a column."""
    maps = _maps(shape, 2, False, seed=sum(shape) + pairs)
    nat.call("si_smooth_set_pairs", pairs)
    try:
        for update in ("f32", "ref_f64"):
            got = _run(maps, 3, update, hits=False)
            assert np.array_equal(got.view(np.uint32), O.smooth(maps, 3, update).view(np.uint32)), update
    finally:
        nat.call("si_smooth_set_pairs", 1)


def test_wait_limit_runs_out_and_reports(cuda):
    """With the wait limit at 0 spins every TMA wait of the smoothing kernels
    gives up at once; the kernels let their copies land, record the status
    and return. si_smooth_status reports it (and clears it); with the default
    limit restored the same call is correct again on the same context."""
    maps = _maps((20, 16, 70), 2, False, seed=2)
    nat.call("si_set_wait_limit", 0)
    try:
        nol, Zc, Yc, Xc = maps.shape
        tmp0, tmp1 = smooth_buffers(Zc, Yc, Xc, cuda)
        t = torch.from_numpy(maps).to(cuda)
        st = torch.cuda.current_stream().cuda_stream
        nat.call("si_smooth_f32", t.data_ptr(), tmp0.data_ptr(), tmp1.data_ptr(), nol, Zc, Yc, Xc, 3, 0, st)
        status = ctypes.c_int(0)
        rc = nat.lib().si_smooth_status(ctypes.byref(status), ctypes.c_void_p(st))
        assert rc == 2 and status.value == 1
        rc = nat.lib().si_smooth_status(ctypes.byref(status), ctypes.c_void_p(st))
        assert rc == 0 and status.value == 0  # cleared
    finally:
        nat.call("si_set_wait_limit", -1)
    got = _run(maps, 3, "f32", hits=False)
    assert np.array_equal(got, O.smooth(maps, 3, "f32"))
