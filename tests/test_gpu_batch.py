"""Batched smart interpolation: every volume's result equals the single-volume
call and the oracle, bit for bit, whatever the tuner or the graph capture do."""
import contextlib
import io

import numpy as np
import pytest

import oracle as O
from biomedisa_gb300 import _native as nat
from biomedisa_gb300 import smart_interpolation, smart_interpolation_batch
from biomedisa_gb300.synthetic import batch_volumes, plain_volume

pytestmark = pytest.mark.gpu


def _volumes():
    vols = batch_volumes(seed=3, count=5, lo=(20, 22, 24), hi=(34, 40, 38))
    imgs = [v[0] for v in vols]
    labs = [v[1] for v in vols]
    # mix in uint8 volumes of another size (uint8 and float records in one batch)
    for s in (8, 9):
        img, lab, _ = plain_volume(seed=s, shape=(26 + s, 30, 28), z_every=4, semi=(5, 10))
        imgs.append(img)
        labs.append(lab)
    return imgs, labs


@pytest.mark.parametrize("graph,device_loop,pairs", [(True, 1, 1), (False, 1, 1), (True, 0, 1), (True, 1, 0)],
                         ids=["graph", "no_graph", "host_loop", "one_walker_per_thread"])
def test_batch_equals_single_and_oracle(graph, device_loop, pairs, cuda, tmp_path, monkeypatch):
    """Also with the host-side sweep loop and with one walker per thread
    (the defaults are the device loop and walker pairs)."""
    monkeypatch.setenv("SI_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    imgs, labs = _volumes()
    kw = dict(nbrw=2, sorw=90, smooth=3, uncertainty=True, return_hits=True)
    rep = {}
    nat.call("si_walk_sorted_set_loop", device_loop)
    nat.call("si_walk_sorted_set_pairs", pairs)
    try:
        got = smart_interpolation_batch(imgs, labs, rng_seed=11, graph=graph, report=rep, **kw)
    finally:
        nat.call("si_walk_sorted_set_loop", 1)
        nat.call("si_walk_sorted_set_pairs", 1)
    assert rep["sweeps"] > 0 and rep["sort_edge"] > 0
    assert len(got) == len(imgs)
    for img, lab, g in zip(imgs, labs, got):
        single = smart_interpolation(img, lab, rng_seed=11, **kw)
        exp = O.smart_interpolation(img, lab, nbrw=2, sorw=90, smooth_iters=3, uncertainty_map=True,
                                    return_hits=True, key=11)
        assert set(g) == set(single) == {"regular", "smooth", "uncertainty", "hits"}
        for k in g:
            assert np.array_equal(g[k], single[k]), k
            assert np.array_equal(g[k], exp[k]), k


def test_batch_tuner_cache_and_errors(cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("SI_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    imgs, labs = _volumes()
    imgs = imgs[:3] + [imgs[3]]
    labs = labs[:3] + [labs[3][:, :, :5]]  # shape mismatch -> None, like the reference's error
    rep1, rep2 = {}, {}
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        r1 = smart_interpolation_batch(imgs, labs, nbrw=1, sorw=60, rng_seed=5, report=rep1)
        r2 = smart_interpolation_batch(imgs, labs, nbrw=1, sorw=60, rng_seed=5, report=rep2)
    assert "same x,y,z-dimensions" in buf.getvalue()
    assert r1[3] is None and r2[3] is None
    assert rep1.get("cached") is False and rep2.get("cached") is True
    assert (tmp_path / "tune.json").exists()
    for a, b in zip(r1[:3], r2[:3]):
        assert np.array_equal(a["regular"], b["regular"])
