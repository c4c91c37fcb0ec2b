"""GPU parity of the active-contour post-processing (si_acwe_*, through the
C-ABI and the package's activeContour / smart_interpolation(acwe=True))
against the reference's own outputs (tests/golden/ref_acwe.npz) and the
oracle (oracle/acwe_oracle.py).

'acwe' (evolution, erosion, dilation, curvop) is integer and binary32/64
comparison work: bit-exact. 'refined' decides each band voxel by comparing two
Gaussian likelihoods; the device takes the classes' standard deviations from
band histograms and evaluates exp() with CUDA's libm, so a decision may
differ from the reference's only where the two likelihoods agree to a
relative 1e-9 (none of these inputs has such a voxel: the tests require
equality everywhere else and report the rest)."""
import numpy as np
import pytest
import torch

import acwe_oracle as A
from biomedisa_gb300 import _native as nat
from biomedisa_gb300 import smart_interpolation
from biomedisa_gb300.active_contour import activeContour
from biomedisa_gb300.synthetic import blob_volume, plain_volume
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = ("u8", "f32_alpha", "crop_x", "nozero", "edges")
NEAR_TIE = 1e-9


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _refined_ok(got, exp, margin):
    bad = got != exp
    return not np.any(bad & (margin > NEAR_TIE)), int(np.count_nonzero(bad))


@pytest.fixture(scope="module")
def fixtures():
    return np.load(GOLDEN / "ref_acwe.npz")


@pytest.mark.parametrize("name", CASES)
def test_acwe_matches_reference_outputs(fixtures, name, cuda):
    img, lab = fixtures[f"{name}_image"], fixtures[f"{name}_labels"]
    alpha, smooth, steps = fixtures[f"{name}_params"]
    got = activeContour(img, lab, alpha, int(smooth), int(steps))
    assert np.array_equal(got, fixtures[f"{name}_acwe"])


@pytest.mark.parametrize("name", CASES)
def test_refined_matches_reference_outputs(fixtures, name, cuda):
    img, lab = fixtures[f"{name}_image"], fixtures[f"{name}_labels"]
    got = activeContour(img, lab, simple=True)
    assert np.array_equal(got, fixtures[f"{name}_refined"])


def _tie_volume(rng, shape, nol, block=2):
    lab = rng.integers(0, nol, size=shape).astype(np.uint8)
    lab = np.repeat(np.repeat(lab[:, ::block, ::block], block, axis=1), block, axis=2)[:, : shape[1], : shape[2]]
    img = (rng.integers(0, 5, size=shape) * 37).astype(np.uint8)
    return img, np.ascontiguousarray(lab)


STENCIL_SHAPES = [(1, 4, 5), (2, 3, 3), (3, 3, 3), (4, 9, 33), (17, 10, 40), (18, 17, 65), (33, 9, 31)]


@pytest.mark.parametrize("shape", STENCIL_SHAPES, ids=[f"{z}x{y}x{x}" for z, y, x in STENCIL_SHAPES])
def test_stencil_passes_bit_exact(shape, cuda):
    """One evolution, erosion and dilation pass and curvop through the C-ABI,
    on tie-heavy label volumes (equal label means, many boundaries), against
    the oracle. Shapes straddle the kernels' 32 x 8 x 16 tiles."""
    rng = np.random.default_rng(sum(shape))
    img, lab = _tie_volume(rng, shape, 5)
    mean = A.label_means(img, lab)
    n = lab.size
    D = torch.from_numpy(img.ravel()).to(cuda)
    L = torch.from_numpy(lab.ravel()).to(cuda)
    out = torch.empty_like(L)
    sums = torch.zeros(512, dtype=torch.int64, device=cuda)
    nat.call("si_acwe_label_sums", D.data_ptr(), L.data_ptr(), n, sums.data_ptr(), _stream())
    s = sums.cpu().numpy()
    cnt = np.bincount(lab.ravel(), minlength=256)
    tot = np.bincount(lab.ravel(), weights=img.ravel().astype(np.float64), minlength=256)
    assert np.array_equal(s[:256], cnt) and np.array_equal(s[256:], tot.astype(np.int64))
    for alpha in (1.0, 0.45, 3.0):
        nat.call("si_acwe_evolution", L.data_ptr(), D.data_ptr(), sums.data_ptr(), alpha, *shape, out.data_ptr(),
                 _stream())
        exp = A.evolution(mean, lab, img, alpha)
        assert np.array_equal(out.cpu().numpy().reshape(shape), exp), alpha
    for label in range(5):
        for erode in (1, 0):
            nat.call("si_acwe_morph", L.data_ptr(), *shape, label, erode, out.data_ptr(), _stream())
            exp = A.erosion(lab, label) if erode else A.dilation(lab, label)
            assert np.array_equal(out.cpu().numpy().reshape(shape), exp), (label, erode)
        for steps in (1, 2, 3):
            Lc = L.clone()
            tmp = torch.empty_like(Lc)
            nat.call("si_acwe_curvop", Lc.data_ptr(), tmp.data_ptr(), *shape, label, steps, _stream())
            assert np.array_equal(Lc.cpu().numpy().reshape(shape), A.curvop(lab, steps, label)), (label, steps)


@pytest.mark.parametrize("kind", ["points", "blobs"])
@pytest.mark.parametrize("shape", [(12, 20, 40), (30, 25, 33), (6, 41, 70)], ids=["12x20x40", "30x25x33", "6x41x70"])
def test_chamfer_band_equals_reference_scan(kind, shape, cuda):
    """si_acwe_chamfer_band (Jacobi relaxation) against the reference's
    forward/backward raster scan (the oracle's restatement): distance <= 10
    agrees on every voxel off the crop's first and last planes, rows and
    columns (where, in a real crop, padding or voxels 100 away from any
    label sit), and those rows and columns are never band. Labels are kept
    off that shell, as in a padded crop."""
    rng = np.random.default_rng(sum(shape) + len(kind))
    if kind == "points":
        lab = (rng.random(shape) < 0.002).astype(np.uint8) * 3
    else:
        Z, Y, X = shape
        _, blobs = blob_volume(shape, sum(shape), [1, 2], [(Z / 2, Y / 3, X / 2), (Z / 3, Y / 2, X / 4)],
                               [(Z / 4, 6, 8), (2, 4, 3)], 5.0)
        lab = blobs.astype(np.uint8)
    lab[0] = lab[-1] = 0
    lab[:, 0] = lab[:, -1] = 0
    lab[:, :, 0] = lab[:, :, -1] = 0
    assert lab.any()
    _, band = A.chamfer_band(lab)
    n = lab.size
    L = torch.from_numpy(lab.ravel()).to(cuda)
    d = torch.empty(n, dtype=torch.float32, device=cuda)
    t = torch.empty_like(d)
    nat.call("si_acwe_dist_init", L.data_ptr(), n, d.data_ptr(), _stream())
    nat.call("si_acwe_chamfer_band", d.data_ptr(), t.data_ptr(), *shape, _stream())
    got = d.cpu().numpy().reshape(shape) <= 10
    core = (slice(1, -1),) * 3
    assert np.array_equal(got[core], band[core]), int(np.count_nonzero(got[core] != band[core]))
    assert not got[:, 0].any() and not got[:, -1].any() and not got[:, :, 0].any() and not got[:, :, -1].any()
    assert 0 < band[core].mean() < 1  # the band neither empty nor everything


RANDOM = [((12, 14, 16), np.uint8, 1.0, 1, 3), ((20, 30, 41), np.float32, 0.7, 2, 2), ((7, 9, 230), np.uint16, 1.0,
          0, 2), ((3, 40, 36), np.int16, 2.2, 3, 1), ((2, 6, 7), np.uint8, 1.0, 1, 2)]


@pytest.mark.parametrize("shape,dtype,alpha,smooth,steps", RANDOM, ids=[f"{c[0]}-{np.dtype(c[1]).name}" for c in RANDOM])
def test_active_contour_matches_oracle(shape, dtype, alpha, smooth, steps, cuda):
    """activeContour in both modes on blob volumes of several dtypes (the
    image conversion img_to_uint8 on the device), with long axes that engage
    the +-100 crop."""
    Z, Y, X = shape
    cz, cy, cx = Z / 2, Y / 2, X / 2
    img, lab = blob_volume(shape, Z * Y + X, [1, 3, 4], [(cz, cy, cx), (cz, cy / 2, cx / 3), (cz / 2, cy, cx * 0.7)],
                           [(max(Z / 3, 1), Y / 4, min(X / 5, 12)), (max(Z / 4, 1), Y / 5, 4),
                            (max(Z / 4, 1), Y / 6, 3)], 16.0, dtype=np.float32)
    if dtype == np.uint8:
        img = np.clip(img, 0, 255).astype(np.uint8)
    elif dtype != np.float32:
        img = (img * 7).astype(dtype)
    lab = lab.astype(np.uint8)
    got = activeContour(img, lab, alpha, smooth, steps)
    assert np.array_equal(got, A.active_contour(img, lab, alpha, smooth, steps))
    got = activeContour(img, lab, simple=True)
    exp, margin = A.active_contour(img, lab, simple=True, margins=True)
    ok, nbad = _refined_ok(got, exp, margin)
    assert ok, nbad


def test_only_ignore_and_big_labels(cuda):
    """pre_processing's label handling before the contour: ``only`` keeps the
    listed labels, ``ignore`` drops labels, values > 255 become 0."""
    img, lab = blob_volume((10, 12, 14), 7, [1, 2, 6], [(5, 6, 7), (3, 3, 3), (7, 9, 10)], [(3, 3, 4), (2, 2, 2),
                           (2, 2, 3)], 10.0)
    lab = lab.astype(np.int32)
    lab[0, 0, :4] = 300
    for kw, keep in (({"only": "1,6"}, (1, 6)), ({"ignore": "2"}, (1, 6)), ({}, (1, 2, 6))):
        ref_lab = np.where(np.isin(lab, keep), lab, 0).astype(np.uint8)
        got = activeContour(img, lab, 1.0, 1, 2, **kw)
        assert np.array_equal(got, A.active_contour(img, ref_lab, 1.0, 1, 2)), kw
        got = activeContour(img, lab, simple=True, **kw)
        exp, margin = A.active_contour(img, ref_lab, simple=True, margins=True)
        assert _refined_ok(got, exp, margin)[0], kw
    with pytest.raises(ValueError, match="negative"):
        activeContour(img, np.where(lab == 2, -1, lab), 1.0, 1, 1)
    assert activeContour(img, np.zeros_like(lab), 1.0, 1, 1) is None


def _reference_image(img, crop):
    """The image smart_interpolation hands activeContour (rw_small.py:247-249):
    the normalised working image inside the interpolation's crop, 0 outside."""
    if img.dtype == np.uint8:
        w = img.copy()
    else:
        w = img.astype(np.float32)
        w -= np.amin(w)
        w /= np.amax(w)
        w *= np.float32(255.0)
    out = np.zeros_like(w)
    z0, z1, y0, y1, x0, x1 = crop  # padded coordinates
    sl = tuple(slice(max(a - 1, 0), b - 1) for a, b in ((z0, z1), (y0, y1), (x0, x1)))
    out[sl] = w[sl]
    return out


@pytest.mark.parametrize("case", ["u8", "f32_crop"])
def test_pipeline_acwe_and_refined(case, cuda):
    """smart_interpolation(acwe=True) returns 'acwe' and 'refined' equal to the
    oracle's activeContour on the regular result and the image the reference
    passes (zero outside the interpolation's crop)."""
    if case == "u8":
        img, lab, _ = plain_volume(seed=8, shape=(30, 34, 38), z_every=6, semi=(6, 12))
        crop = (0, 32, 0, 36, 0, 40)
    else:
        # labels in the middle of a long x axis: the interpolation's crop
        # leaves zeros at both ends of x
        img, lab, _ = plain_volume(seed=9, shape=(24, 26, 280), z_every=5, semi=(5, 9))
        img = img.astype(np.float32) * 3.3 - 17.0
        lab[:, :, :110] = 0
        lab[:, :, 170:] = 0
        nz = np.nonzero(lab)
        x0, x1 = int(nz[2].min()) + 1, int(nz[2].max()) + 1  # padded coordinates
        crop = (0, 26, 0, 28, max(x0 - 100, 0), min(x1 + 100, 282))
        assert crop[4] > 0 and crop[5] < 282
    res = smart_interpolation(img, lab, nbrw=2, sorw=200, acwe=True, acwe_alpha=1.0, acwe_smooth=1, acwe_steps=3)
    ref_img = _reference_image(img, crop)
    exp = A.active_contour(ref_img, res["regular"], 1.0, 1, 3)
    assert np.array_equal(res["acwe"], exp)
    exp, margin = A.active_contour(ref_img, res["regular"], simple=True, margins=True)
    ok, nbad = _refined_ok(res["refined"], exp, margin)
    assert ok, nbad
    assert np.count_nonzero(res["acwe"] != res["regular"]) > 0
