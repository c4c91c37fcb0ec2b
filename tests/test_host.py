"""Host-side planning logic (no GPU): label plans, crops, the large path's
slice list, volume groups of the batched walk, slot permutations of the
surrogate's training."""
import numpy as np
import pytest

from biomedisa_gb300 import interpolation as I
from biomedisa_gb300.batch import volume_groups
import oracle as O


def test_large_slice_list_matches_oracle():
    rng = np.random.default_rng(0)
    for _ in range(20):
        zs = np.sort(rng.choice(60, size=rng.integers(1, 25), replace=False))
        lab = np.zeros((60, 4, 4), np.int32)
        lab[zs, 1, 1] = 1
        sl = np.asarray([(0, int(z)) for z in zs], np.int32)
        got = [int(z) for _, z in I.large_slice_list(sl).tolist()]
        assert got == O.read_labeled_slices_large(lab)


def test_large_slice_list_keeps_z_only():
    sl = np.asarray([(0, 2), (0, 4), (0, 8), (1, 3), (2, 5)], np.int32)
    assert I.large_slice_list(sl).tolist() == [[0, 2], [0, 8]]


def test_volume_groups_cover_in_order():
    rng = np.random.default_rng(1)
    for _ in range(50):
        seeds = rng.integers(0, 5_000_000, size=rng.integers(1, 40)).tolist()
        groups = volume_groups(seeds, 10, group_walks=1 << 25)
        flat = [k for a, b in groups for k in range(a, b)]
        assert flat == list(range(len(seeds)))
        for a, b in groups[:-1]:
            assert sum(seeds[a:b]) * 10 >= 1 << 25
            assert sum(seeds[a:b - 1]) * 10 < 1 << 25


def test_plan_labels_only_ignore():
    hist = np.zeros(258, np.int64)
    hist[[0, 1, 2, 5]] = 10
    hist[256] = 3  # negatives
    p = I.plan_labels(hist, only="1,5")
    assert p.all_labels.tolist() == [0, 1, 5]
    assert p.slot_lut[2] == 0 and p.slot_lut[5] == 2 and p.slot_lut[1] == 1
    q = I.plan_labels(hist, ignore="2")
    assert q.all_labels.tolist() == [0, 1, 5] and q.slot_lut[2] == 0


def test_plan_crop_matches_predict_blocksize():
    rng = np.random.default_rng(2)
    for _ in range(10):
        shape = tuple(int(v) for v in rng.integers(5, 300, 3))
        lab = np.zeros(shape, np.int32)
        z = rng.integers(0, shape[0]); y0, y1 = sorted(rng.integers(0, shape[1], 2)); x0, x1 = sorted(
            rng.integers(0, shape[2], 2))
        lab[z, y0:y1 + 1, x0:x1 + 1] = 1
        padded = np.pad(lab, 1)
        az, bz, ay, by, ax, bx = O.predict_blocksize(padded)
        flags = [np.zeros(s + 2, np.uint8) for s in shape]
        flags[0][z + 1] = 1
        bbox = (z + 1, z + 1, y0 + 1, y1 + 1, x0 + 1, x1 + 1)
        cp = I.plan_crop(shape, bbox, flags, False)
        assert (cp.cz0, cp.cz0 + cp.Zc, cp.cy0, cp.cy0 + cp.Yc, cp.cx0, cp.cx0 + cp.Xc) == (az, bz, ay, by, ax, bx)
        assert cp.slice_list.tolist() == [[0, z + 1 - az]]


def test_slot_permutation_keeps_slot_zero():
    from biomedisa_gb300.surrogate import MAX_SLOTS, _slot_permutation
    rng = np.random.default_rng(3)
    for nol in range(1, MAX_SLOTS + 1):
        src, dst = _slot_permutation(rng, nol)
        assert dst[0] == 0 and len(set(dst.tolist())) == nol
        new = np.arange(16)[src]
        for k in range(nol):
            assert new[3 + dst[k]] == 3 + k


def test_out_of_memory_degrades_like_the_reference(capsys):
    """Smoothing and uncertainty buffers: a device out-of-memory error prints
    the reference's warning and drops that output (rw_small.py:147-149,
    181-183); other errors propagate."""
    import torch

    def oom():
        raise torch.cuda.OutOfMemoryError("forced")

    assert I._or_warn_on_oom(oom, I.SMOOTH_OOM_WARNING) is None
    assert capsys.readouterr().out.strip() == I.SMOOTH_OOM_WARNING
    assert I._or_warn_on_oom(lambda: 7, I.UNCERTAINTY_OOM_WARNING) == 7
    assert capsys.readouterr().out == ""

    def other():
        raise ValueError("not memory")

    with pytest.raises(ValueError):
        I._or_warn_on_oom(other, I.SMOOTH_OOM_WARNING)


def test_autotune_cache_round_trip(tmp_path, monkeypatch):
    from biomedisa_gb300 import autotune as A

    monkeypatch.setenv("SI_AUTOTUNE_CACHE", str(tmp_path / "sub" / "tune.json"))
    assert A._load() == {}
    A._store("k1", [6, 32])
    A._store("k2", [8, 64])
    assert A._load() == {"k1": [6, 32], "k2": [8, 64]}
    assert sorted(p.name for p in (tmp_path / "sub").iterdir()) == ["tune.json"]  # no temporary left behind
    (tmp_path / "sub" / "tune.json").write_text("{not json")
    assert A._load() == {}  # a damaged cache is ignored (the workload is tuned again)


def test_surrogate_checkpoint_round_trip(tmp_path):
    """save/load keep weights, biases, AdamW moments and the step count; a
    weights-only checkpoint loads with zero moments and step count 0; a
    partial set of moments and a different shape are refused. (The network is built on the CPU device here: no kernel runs.)"""
    import torch

    from biomedisa_gb300 import surrogate as SG

    a = SG.SurrogateNet(device="cpu", seed=1)
    g = torch.Generator().manual_seed(5)
    for c in a.convs:
        for m in ("mw", "vw", "mb", "vb"):
            getattr(c, m).copy_(torch.rand(getattr(c, m).shape, generator=g))
    a.step_count = 17
    path = tmp_path / "net.pt"
    SG.save(a, path)
    b = SG.load(path, device="cpu")
    assert b.step_count == 17 and (b.channels, b.dilations) == (a.channels, a.dilations)
    for ca, cb in zip(a.convs, b.convs):
        for f in ("w", "b", "wb", "mw", "vw", "mb", "vb"):
            assert torch.equal(getattr(ca, f), getattr(cb, f)), f
    sd = a.state_dict()
    for m in ("mw", "vw", "mb", "vb"):
        del sd[m]
    c = SG.SurrogateNet(device="cpu", seed=2)
    c.load_state_dict(sd)
    assert torch.equal(c.convs[3].w, a.convs[3].w) and not c.convs[3].mw.any()
    assert c.step_count == 0  # weights only: AdamW restarts, bias correction included
    partial = a.state_dict()
    del partial["vb"]
    with pytest.raises(ValueError):
        SG.SurrogateNet(device="cpu", seed=2).load_state_dict(partial)
    d = SG.SurrogateNet(channels=32, device="cpu")
    with pytest.raises(ValueError):
        d.load_state_dict(a.state_dict())


def test_autotune_store_concurrent_threads(tmp_path, monkeypatch):
    """Threads of one process storing autotune entries at once keep every
    entry and leave no temporary files behind."""
    import threading

    from biomedisa_gb300 import autotune as AT

    path = tmp_path / "cache.json"
    monkeypatch.setenv("SI_AUTOTUNE_CACHE", str(path))
    threads = [threading.Thread(target=AT._store, args=(f"k{i}", {"sort_edge": 6, "sweep_steps": i}))
               for i in range(16)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    data = AT._load()
    assert sorted(data) == sorted(f"k{i}" for i in range(16))
    assert [p.name for p in tmp_path.iterdir()] == ["cache.json"]
