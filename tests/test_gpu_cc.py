"""clean / fill on the device (si_clean, si_fill through
biomedisa_gb300.postprocess) against the reference's own outputs and the
oracle: bit-exact label volumes."""
import numpy as np
import pytest
import torch

import cc_oracle as C
from biomedisa_gb300 import postprocess as P
from biomedisa_gb300 import synthetic as S
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _dev(a, cuda):
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def test_reference_fixtures(cuda):
    z = np.load(GOLDEN / "ref_cc.npz")
    names = sorted(k[:-3] for k in z.files if k.endswith("_in"))
    for n in names:
        v = _dev(z[f"{n}_in"], cuda)
        for thr in (0.1, 0.5):
            assert np.array_equal(P.clean(v, thr).cpu().numpy(), z[f"{n}_clean_{thr}"]), (n, thr)
        for thr in (0.9, 0.3):
            assert np.array_equal(P.fill(v, thr).cpu().numpy(), z[f"{n}_fill_{thr}"]), (n, thr)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_volumes_against_oracle(seed, cuda):
    """Interpolation-like volumes with speckle and holes, 64 x 70 x 90."""
    rng = np.random.default_rng(seed)
    truth = np.zeros((64, 70, 90), np.uint8)
    S._phases(rng, truth, 6, size_frac=(0.1, 0.3))
    noise = rng.random(truth.shape)
    vol = truth.copy()
    sel = noise < 0.03
    vol[sel] = rng.integers(0, 7, size=int(sel.sum()))
    v = _dev(vol, cuda)
    for thr in (0.1, 0.9):
        assert np.array_equal(P.clean(v, thr).cpu().numpy(), C.clean(vol, thr))
    for thr in (0.9, 0.2):
        assert np.array_equal(P.fill(v, thr).cpu().numpy(), C.fill(vol, thr))


def test_edge_cases(cuda):
    """A label that fills its whole box, a vanished label, one label only, an
    empty volume, a volume without label 0."""
    v = np.zeros((8, 9, 10), np.uint8)
    v[2:5, 2:5, 2:5] = 3  # the label outweighs its complement inside its box
    v[0, 0, 0] = 3
    v[6, 7, 8] = 5
    for thr in (0.1, 0.9):
        assert np.array_equal(P.fill(_dev(v, cuda), thr).cpu().numpy(), C.fill(v, thr))
        assert np.array_equal(P.clean(_dev(v, cuda), thr).cpu().numpy(), C.clean(v, thr))
    nest = np.zeros((12, 12, 12), np.uint8)
    nest[2:10, 2:10, 2:10] = 1
    nest[4:8, 4:8, 4:8] = 0
    nest[5:7, 5:7, 5:7] = 2
    assert np.array_equal(P.fill(_dev(nest, cuda), 0.9).cpu().numpy(), C.fill(nest, 0.9))
    for vol in (np.zeros((5, 6, 7), np.uint8), np.full((5, 6, 7), 4, np.uint8),
                np.random.default_rng(3).integers(2, 5, (9, 10, 11)).astype(np.uint8)):
        assert np.array_equal(P.fill(_dev(vol, cuda), 0.9).cpu().numpy(), C.fill(vol, 0.9))
        assert np.array_equal(P.clean(_dev(vol, cuda), 0.1).cpu().numpy(), C.clean(vol, 0.1))


def test_smart_interpolation_post_keys(cuda):
    """clean / fill through the drop-in call: result keys and values as
    rw_small.py:223-243 derives them from 'regular' and 'smooth'."""
    from biomedisa_gb300 import smart_interpolation
    img, lab, _ = S.plain_volume(seed=6, shape=(48, 52, 56), z_every=6, semi=(8, 18))
    r = smart_interpolation(img, lab, nbrw=4, sorw=300, smooth=5, clean=0.1, fill=0.9)
    for k in ("regular", "smooth", "cleaned", "smooth_cleaned", "filled", "cleaned_filled"):
        assert k in r, k
    assert np.array_equal(r["cleaned"], C.clean(r["regular"], 0.1))
    assert np.array_equal(r["smooth_cleaned"], C.clean(r["smooth"], 0.1))
    assert np.array_equal(r["filled"], C.fill(r["regular"], 0.9))
    assert np.array_equal(r["cleaned_filled"], C.cleaned_filled(r["cleaned"], r["filled"], r["regular"]))
