"""GPU parity: the CUDA path (through the C ABI) against the oracle, bit for bit.

Every output of smart_interpolation — regular labels, smoothed labels,
uncertainty, hit maps — and the intermediate seeds, label plan and slice
flags must equal the oracle's on the same seeded inputs."""
import contextlib
import io

import numpy as np
import pytest
import torch

import oracle as O
from biomedisa_gb300 import smart_interpolation, walk
from biomedisa_gb300 import interpolation as I
from biomedisa_gb300.synthetic import plain_volume, sparse_labels

pytestmark = pytest.mark.gpu


def _large_allx_case():
    """Labels on z-slices 3 and 11, y-slice 15 and x-slice 400 of a
    16 x 22 x 460 volume (planes wider than the adaptive window), a -1 patch."""
    lab = np.zeros((16, 22, 460), np.int32)
    for z in (3, 11):
        lab[z, :, :300] = 1
        lab[z, :, 300:450] = 2
    lab[11, 6:10, 40:70] = -1
    lab[:, 15, :300] = 1
    lab[:, 15, 300:420] = 2
    lab[:, :, 400] = 2
    lab[4:9, 5:12, 400] = 1
    img = (np.random.default_rng(6).normal(90, 20, lab.shape) + 60 * (lab == 2)).clip(0, 255).astype(np.uint8)
    return lab, img


def _cases():
    img, lab, truth = plain_volume(seed=1, shape=(40, 36, 34), z_every=5, semi=(6, 12))
    base = dict(nbrw=3, sorw=70, smooth=3, uncertainty=True, return_hits=True)
    yield "u8", img, lab, base
    yield "u8_packed_walker", img, lab, dict(base, walker="packed")
    yield "u8_tiles_walker", img, lab, dict(base, walker="tiles")
    yield "u16", img.astype(np.uint16) * 3 + 7, lab, base
    yield "i8_denoise", (img.astype(np.int16) - 128).astype(np.int8), lab, dict(base, denoise=True, smooth=0)
    yield "f32_denoise", img.astype(np.float32) * 0.37 - 5.0, lab, dict(base, denoise=True, smooth=2)
    yield "f64", img.astype(np.float64) / 7.0, lab, dict(base, smooth=1)
    yield "u8_labels_u8", img, lab.astype(np.uint8), base
    yield "u8_labels_i64", img, lab.astype(np.int64), base
    rng = np.random.default_rng(5)
    img2, _, truth2 = plain_volume(seed=2, shape=(34, 38, 36), z_every=4, semi=(6, 12))
    t2 = truth2.astype(np.int32)
    t2[(t2 == 0) & (rng.random(t2.shape) < 0.02)] = 3
    t2[5:9, 5:12, 5:12] = 4
    lab2 = sparse_labels(t2, z_every=4)
    lab2[8, 2:6, 2:6] = -1
    lab2[12, 30:33, 30:33] = 300
    yield "neg_big", img2, lab2, dict(base, smooth=2)
    yield "only", img2, lab2, dict(base, only="1,2", smooth=0)
    yield "ignore", img2, lab2, dict(base, ignore="3", smooth=0)
    img3, _, truth3 = plain_volume(seed=4, shape=(38, 40, 36), z_every=6, semi=(7, 13))
    lab3 = sparse_labels(truth3.astype(np.int32), z_every=6, y_every=9, x_every=9)
    yield "allaxis_u8", img3, lab3, dict(base, allaxis=True, smooth=2)
    yield "allaxis_u8_packed", img3, lab3, dict(base, allaxis=True, smooth=0, walker="packed")
    yield "allaxis_u16", img3.astype(np.uint16) * 5, lab3, dict(base, allaxis=True, smooth=0)
    # labels near the volume border (crop clamped), odd sizes
    img4, _, truth4 = plain_volume(seed=9, shape=(17, 23, 29), z_every=2, semi=(4, 9))
    yield "small_border", img4, sparse_labels(truth4.astype(np.int32), z_every=2), dict(base, smooth=4)
    # a large margin: crop strictly inside the volume (bbox +- 100)
    big = np.full((30, 260, 250), 60, np.uint8)
    big += np.random.default_rng(3).integers(0, 9, big.shape, dtype=np.uint8)
    tb = np.zeros(big.shape, np.int32)
    tb[:, 120:140, 115:135] = 1
    big[tb == 1] = 190
    lb = sparse_labels(tb, z_every=3)
    lb[lb == 0] = 0
    lb[::3, 110:150, 105:145] = np.where(tb[::3, 110:150, 105:145] == 1, 1, 2)
    yield "inner_crop", big, lb, dict(base, nbrw=1, sorw=40, smooth=1)
    # the reference large path's seed set (slice skipping, label box, adaptive seeds)
    yield "large_seeding_inner", big, lb, dict(base, nbrw=1, sorw=40, smooth=2, seeding="large")
    yield "large_seeding_neg_ignore", img2, lab2, dict(base, smooth=2, ignore="3", seeding="large")
    ll = np.zeros((18, 26, 240), np.int32)
    for z in (2, 5, 9, 13):
        ll[z, 2:24, 3:120] = 1
        ll[z, 2:24, 120:230] = 2
    ll[9, 10:14, 40:60] = -1
    ll[15] = 1
    il = (np.random.default_rng(4).normal(90, 20, ll.shape) + 60 * (ll == 2)).clip(0, 255).astype(np.uint8)
    yield "large_seeding_wide", il, ll, dict(base, nbrw=2, sorw=40, smooth=2, seeding="large")
    # the all-axis large path's seed set (every slice with a positive label on
    # each axis, one box per axis, adaptive seeds in slice coordinates)
    yield "large_allx_u8", img3, lab3, dict(base, allaxis=True, smooth=2, seeding="large")
    la, ia = _large_allx_case()
    yield "large_allx_wide", ia, la, dict(base, nbrw=2, sorw=40, allaxis=True, smooth=2, seeding="large")
    lb2 = np.zeros(big.shape, np.int32)
    for z in range(0, 30, 4):
        lb2[z, 110:150, 105:145] = np.where(tb[z, 110:150, 105:145] == 1, 1, 2)
    for y in (118, 131):
        lb2[1:29, y, 100:150] = np.where(tb[1:29, y, 100:150] == 1, 1, 2)
    lb2[2:28, 112:148, 126] = np.where(tb[2:28, 112:148, 126] == 1, 1, 2)
    lb2[6:9, 120:124, 126] = -1
    yield "large_allx_inner", big, lb2, dict(base, nbrw=1, sorw=40, allaxis=True, smooth=1, seeding="large")


CASES = list(_cases())


@pytest.mark.parametrize("name,img,lab,kw", CASES, ids=[c[0] for c in CASES])
def test_pipeline_bit_exact(name, img, lab, kw, cuda):
    key = 0x1234_5678_9ABC_DEF0
    got = smart_interpolation(img, lab, rng_seed=key, **kw)
    exp = O.smart_interpolation(
        img, lab, nbrw=kw["nbrw"], sorw=kw["sorw"], smooth_iters=kw.get("smooth", 0),
        allaxis=kw.get("allaxis", False), uncertainty_map=kw.get("uncertainty", False),
        return_hits=kw.get("return_hits", False), denoise=kw.get("denoise", False), only=kw.get("only", "all"),
        ignore=kw.get("ignore", "none"), key=key, seeding=kw.get("seeding", "plain"))
    assert set(got) == {k for k in ("regular", "smooth", "uncertainty", "hits") if k in exp}
    for k, v in got.items():
        assert v.dtype == exp[k].dtype and v.shape == exp[k].shape, k
        assert np.array_equal(v, exp[k]), f"{name}: {k} differs in {np.count_nonzero(v != exp[k])} voxels"


def _job(img, lab, **kw):
    d, l = I.normalize_host_dtypes(img, lab)
    ti, tl = I.upload(d, l)
    job = I.DeviceJob(ti, I._IMG_DTYPES[d.dtype], tl, I._LAB_DTYPES[l.dtype], **kw)
    assert job.analyze() is None
    job.prepare()
    return job


@pytest.mark.parametrize("allaxis", [False, True])
def test_seeds_and_plans_bit_exact(allaxis, cuda):
    img, lab, truth = plain_volume(seed=12, shape=(36, 40, 38), z_every=5, semi=(6, 12))
    if allaxis:
        lab = sparse_labels(truth.astype(np.int32), z_every=5, y_every=7, x_every=8)
    job = _job(img, lab, allaxis=allaxis)
    o = O.smart_interpolation(img, lab, nbrw=0, sorw=0, allaxis=allaxis)
    assert list(job.lplan.all_labels) == list(o["allLabels"])
    az, bz, ay, by, ax, bx = o["crop"]
    cp = job.cplan
    assert (cp.cz0, cp.cz0 + cp.Zc, cp.cy0, cp.cy0 + cp.Yc, cp.cx0, cp.cx0 + cp.Xc) == (az, bz, ay, by, ax, bx)
    assert [tuple(e) for e in cp.slice_list.tolist()] == [tuple(e) for e in o["slice_list"]]
    n = int(job.n_seeds.item())
    s = o["seeds"]
    assert n == len(s)
    rec = job.seeds[: n * 16].cpu().numpy().view(np.uint32).reshape(n, 4)
    assert np.array_equal(rec[:, 0], s.pos)
    assert np.array_equal(rec[:, 1], s.c.view(np.uint32))
    assert np.array_equal(rec[:, 2], s.b.view(np.uint32))
    assert np.array_equal(rec[:, 3], s.slot | (s.axis << 8) | (s.label << 16))


def test_walk_invariant_to_launch_shape(cuda):
    """Packed walker under several launch shapes and work orders, and the brick
    walker, give the same hit maps."""
    img, lab, _ = plain_volume(seed=13, shape=(44, 40, 42), z_every=5, semi=(7, 13))
    ref = smart_interpolation(img, lab, nbrw=2, sorw=50, return_hits=True, walker="tiles")["hits"]
    assert ref.sum() > 0
    for k in (1, 7, 64, 1000):
        r = smart_interpolation(img, lab, nbrw=2, sorw=50, return_hits=True, walker="sorted", sweep_steps=k)
        assert np.array_equal(r["hits"], ref)
    for grid, block, order in ((0, 0, 0), (7, 64, 0), (152, 256, 1), (1, 32, 1)):
        r = smart_interpolation(img, lab, nbrw=2, sorw=50, return_hits=True, walk_grid=grid, walk_block=block,
                                walk_order=order, walker="packed")
        assert np.array_equal(r["hits"], ref)


@pytest.mark.parametrize("shape,sorw", [((23, 31, 29), 300), ((12, 70, 9), 500), ((64, 48, 56), 120)])
@pytest.mark.parametrize("walker", ["tiles", "sorted"])
def test_brick_walkers_long_walks_bit_exact(shape, sorw, walker, cuda):
    """Walks much longer than a brick or a sweep (many rounds, odd crop sizes,
    x extent below one brick): tile and sorted walkers == oracle."""
    img, lab, _ = plain_volume(seed=sum(shape), shape=shape, z_every=3, semi=(3, 9))
    key = 77
    got = smart_interpolation(img, lab, nbrw=2, sorw=sorw, return_hits=True, rng_seed=key, walker=walker,
                              sweep_steps=37)
    exp = O.smart_interpolation(img, lab, nbrw=2, sorw=sorw, return_hits=True, key=key)
    assert np.array_equal(got["hits"], exp["hits"])
    assert np.array_equal(got["regular"], exp["regular"])


def test_walk_plugin_seam_matches_oracle(cuda):
    """walk() — the seam a maintainer swaps into rw_small.py — against the oracle."""
    img, lab, _ = plain_volume(seed=14, shape=(30, 32, 28), z_every=4, semi=(5, 10))
    data = np.pad(img, 1)
    l2 = np.pad(lab, 1)
    idx, stack = O.read_labeled_slices(l2)
    child = idx[::2]
    got = walk(data, stack, idx, child, 2, 60, rng_seed=5)
    labels = np.unique(stack)
    labels = labels[labels >= 0]
    seeds = O.extract_seeds(data, l2 * np.isin(np.arange(l2.shape[0]), child)[:, None, None],
                            [(0, k) for k in child], labels)
    exp = O.walk_c(data, seeds, 2, 60, 5, len(labels)).astype(np.float32)
    assert got.dtype == np.float32 and np.array_equal(got, exp)


def test_edge_weight_against_cuda_expf(cuda):
    """Our exp2 weight (oracle == kernel) against CUDA's expf of the same
    argument, where exp(-t) > 1e-30. Both sides round the exponent argument
    twice (ours: c and d2*c; CUDA's: div1 and d2*div1), each a relative 2^-24,
    so the bound is 4 * 2^-24 * t plus 1e-6 for the polynomial and expf."""
    rng = np.random.default_rng(15)
    d2 = rng.integers(0, 65026, 1 << 18).astype(np.float32)
    var = rng.uniform(1, 4000, 1 << 18).astype(np.float32)
    c = O.weight_constant(var)
    w = O.edge_weight(d2, c).astype(np.float64)
    div1 = (np.float32(1.0) / (np.float32(2.0) * var)).astype(np.float32)
    t = torch.from_numpy((-(d2 * div1)).astype(np.float32)).to(cuda)
    e = torch.exp(t).cpu().numpy().astype(np.float64)
    m = e > 1e-30
    tt = -t.cpu().numpy().astype(np.float64)
    bound = 1e-6 + 4 * 2.0**-24 * tt[m]
    assert np.all(np.abs(w[m] - e[m]) / e[m] <= bound)


def test_errors_like_reference(cuda):
    img, lab, _ = plain_volume(seed=16, shape=(20, 20, 20), z_every=3, semi=(4, 8))
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        assert smart_interpolation(img, np.zeros_like(lab)) is None
    assert "No labeled slices found." in buf.getvalue()
    adj = lab.copy()
    adj[1] = adj[0]
    adj[:, 4] = 1
    adj[:, 5] = 1
    with contextlib.redirect_stdout(buf):
        assert smart_interpolation(img, adj, allaxis=True) is None
    assert "At least one empty slice between labels required." in buf.getvalue()
    with contextlib.redirect_stdout(buf):
        assert smart_interpolation(img, lab[:, :, :5]) is None
    assert "same x,y,z-dimensions" in buf.getvalue()


def test_zero_walks_and_tiny_volume(cuda):
    img, lab, _ = plain_volume(seed=17, shape=(3, 3, 3), z_every=1, semi=(1, 2))
    lab = np.zeros((3, 3, 3), np.int32)
    lab[1] = [[0, 1, 0], [1, 1, 0], [0, 0, 2]]
    r = smart_interpolation(img, lab, nbrw=2, sorw=10, return_hits=True, uncertainty=True, smooth=2)
    e = O.smart_interpolation(img, lab, nbrw=2, sorw=10, return_hits=True, uncertainty_map=True, smooth_iters=2,
                              key=I.DEFAULT_RNG_SEED)
    for k in r:
        assert np.array_equal(r[k], e[k]), k
    r0 = smart_interpolation(img, lab, nbrw=0, sorw=10, return_hits=True)
    assert r0["hits"].sum() == 0


def test_large_seeding_box_and_count(cuda):
    """Large-path seeding on the wide case: the in-plane box and the number
    of seeds kept by the adaptive filter equal the oracle's."""
    ll = np.zeros((18, 26, 240), np.int32)
    for z in (2, 5, 9, 13):
        ll[z, 2:24, 3:120] = 1
        ll[z, 2:24, 120:230] = 2
    ll[15] = 1
    ll[15, :, :30] = 0
    il = np.full(ll.shape, 80, np.uint8)
    job = _job(il, ll, seeding="large")
    lab = np.pad(ll, 1)
    az, bz, ay, by, ax, bx = O.predict_blocksize(lab)
    lab = np.ascontiguousarray(lab[az:bz, ay:by, ax:bx])
    idx = O.read_labeled_slices_large(lab)
    llab, box = O.large_labels(lab, idx)
    assert tuple(job.large_box) == tuple(box)
    seeds = O.extract_seeds(np.pad(il, 1)[az:bz, ay:by, ax:bx], llab, [(0, k) for k in idx], O.pre_processing(
        np.pad(ll, 1))[1])
    keep = O.adaptive_seed_mask(llab, seeds)
    assert int(job.n_seeds.item()) == int(keep.sum()) < len(keep)


def test_large_allx_boxes_and_count(cuda):
    """All-axis large-path seeding: the slice list, the per-axis boxes and the
    number of seeds kept by the adaptive filter equal the oracle's."""
    lab, img = _large_allx_case()
    lab[3, 2:20, 290:320] = 3  # a third label inside the z-slices
    job = _job(img, lab, allaxis=True, seeding="large")
    lp = np.pad(lab, 1)
    az, bz, ay, by, ax, bx = O.predict_blocksize(lp)
    lc = np.ascontiguousarray(lp[az:bz, ay:by, ax:bx])
    sl = O.large_allx_slice_list(lc)
    llabs, boxes = O.large_allx_labels(lc, sl)
    for a, box in boxes.items():
        assert tuple(job.large_boxes[a]) == tuple(box), a
    seeds = O.extract_seeds(np.pad(img, 1)[az:bz, ay:by, ax:bx], llabs, sl, O.pre_processing(lp)[1])
    keep = O.adaptive_seed_mask_allx(llabs, seeds)
    assert int(job.n_seeds.item()) == int(keep.sum()) < len(keep)
