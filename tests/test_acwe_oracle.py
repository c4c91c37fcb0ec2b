"""Pins the active-contour oracle (oracle/acwe_oracle.py) to the reference
(CPU): the committed outputs of the reference's own activeContour
(tests/golden/ref_acwe.npz, both modes), and live comparisons with the
reference's evolution / curvop / activeContour where the reference tree is
present (imported with numba's typing restored, oracle/ref_import.py). Also
checks the product's host-side crop arithmetic against the oracle."""
from pathlib import Path

import numpy as np
import pytest

import acwe_oracle as A
from conftest import GOLDEN

CASES = ("u8", "f32_alpha", "crop_x", "nozero", "edges")


@pytest.fixture(scope="module")
def fixtures():
    return np.load(GOLDEN / "ref_acwe.npz")


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_reference_acwe(fixtures, name):
    img, lab = fixtures[f"{name}_image"], fixtures[f"{name}_labels"]
    alpha, smooth, steps = fixtures[f"{name}_params"]
    got = A.active_contour(img, lab, alpha, int(smooth), int(steps))
    assert np.array_equal(got, fixtures[f"{name}_acwe"])
    assert not np.array_equal(got, lab)  # the fixture exercises the contour


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_reference_refined(fixtures, name):
    img, lab = fixtures[f"{name}_image"], fixtures[f"{name}_labels"]
    got, margin = A.active_contour(img, lab, simple=True, margins=True)
    assert np.array_equal(got, fixtures[f"{name}_refined"])
    # no decision of these fixtures is a near-tie (device parity relies on it)
    assert np.min(margin) > 1e-6


def test_dilation_plane_test_never_passes():
    """curvop_numba.py:62-84 counts +1 for every voxel outside the tested
    plane, so its sum is >= 18 and the plane test cannot pass: dilation is a
    plain 27-neighbourhood dilation (the oracle and the kernel rely on it)."""
    P3 = np.zeros((9, 3, 3, 3), np.int32)
    for t, members in enumerate(A.PLANES):
        for i in members:
            dz, dy, dx = A.OFFSETS[i]
            P3[t, dz + 1, dy + 1, dx + 1] = 1
    assert (P3.sum(axis=(1, 2, 3)) == 9).all()
    # the best case for the plane test: every plane voxel differs from the label
    for t in range(9):
        value = sum(0 if P3[t, k, l, m] == 1 else 1 for k in range(3) for l in range(3) for m in range(3))
        assert value == 18


def test_plane_members_match_reference_definition():
    """The nine planes of curvop (curvop_numba.py:125-134), built the way the
    reference indexes _P3, equal the oracle's plane list."""
    P3 = np.zeros((9, 3, 3, 3), dtype=np.int32)
    P3[0, :, :, 1] = 1
    P3[1, :, 1, :] = 1
    P3[2, 1, :, :] = 1
    P3[3, :, [0, 1, 2], [0, 1, 2]] = 1
    P3[4, :, [0, 1, 2], [2, 1, 0]] = 1
    P3[5, [0, 1, 2], :, [0, 1, 2]] = 1
    P3[6, [0, 1, 2], :, [2, 1, 0]] = 1
    P3[7, [0, 1, 2], [0, 1, 2], :] = 1
    P3[8, [0, 1, 2], [2, 1, 0], :] = 1
    for t, members in enumerate(A.PLANES):
        mine = np.zeros((3, 3, 3), np.int32)
        for i in members:
            dz, dy, dx = A.OFFSETS[i]
            mine[dz + 1, dy + 1, dx + 1] = 1
        assert np.array_equal(mine, P3[t]), t


@pytest.mark.parametrize("seed", range(6))
def test_crop_box_matches_oracle(seed):
    from biomedisa_gb300.active_contour import crop_box

    rng = np.random.default_rng(seed)
    shape = tuple(int(v) for v in rng.integers(3, 260, 3))
    lab = np.zeros(shape, np.uint8)
    if seed:
        z, y, x = (int(rng.integers(0, s)) for s in shape)
        lab[z:z + int(rng.integers(1, 4)), y:y + 3, x:x + 5] = 3
    nz = np.nonzero(lab)
    imax = np.iinfo(np.int32).max
    bbox = [imax, -1, imax, -1, imax, -1]
    if nz[0].size:
        bbox = [int(nz[0].min()), int(nz[0].max()), int(nz[1].min()), int(nz[1].max()), int(nz[2].min()),
                int(nz[2].max())]
    z0, z1, y0, y1, x0, x1 = A.crop_box(lab)
    assert crop_box(bbox, shape) == (z0, y0, x0, z1 - z0, y1 - y0, x1 - x0)


def _reference():
    import ref_import

    if not Path(ref_import.REFERENCE_ROOT).is_dir():
        pytest.skip("reference tree not present")
    return ref_import


def _tie_volume(rng, shape, nol):
    """Labels in random blocks (many label boundaries, equal means: ties)."""
    lab = rng.integers(0, nol, size=shape).astype(np.uint8)
    lab = np.repeat(np.repeat(lab[:, ::2, ::2], 2, axis=1), 2, axis=2)[:, : shape[1], : shape[2]]
    img = (rng.integers(0, 4, size=shape) * 40).astype(np.uint8)
    return img, np.ascontiguousarray(lab)


@pytest.mark.parametrize("seed", range(4))
def test_evolution_and_curvop_match_reference_live(seed):
    """The reference's own evolution and curvop (curvop_numba.py) on
    tie-heavy random volumes against the oracle's."""
    ref_import = _reference()
    rng = np.random.default_rng(100 + seed)
    shape = (5, 8, 9) if seed % 2 else (6, 7, 10)
    img, lab = _tie_volume(rng, shape, 4)
    alpha = (1.0, 0.5, 2.0, 0.3)[seed]
    with ref_import.reference_modules():
        import importlib

        cv = importlib.import_module("biomedisa.features.curvop_numba")
        mean = A.label_means(img, lab)
        mean[2] = mean[1]  # force equal costs
        ref_evo = cv.evolution(mean, lab.copy(), img, alpha)
        assert np.array_equal(A.evolution(mean, lab, img, alpha), ref_evo)
        for label in range(4):
            for steps in (1, 2, 3):
                ref_c = cv.curvop(lab.copy(), steps, label, np.arange(4))
                assert np.array_equal(A.curvop(lab, steps, label), ref_c), (label, steps)


@pytest.mark.parametrize("seed", range(3))
def test_active_contour_matches_reference_live(seed):
    """activeContour itself (both modes) on random blob volumes."""
    ref_import = _reference()
    from biomedisa_gb300.synthetic import blob_volume

    rng = np.random.default_rng(200 + seed)
    shape = (9 + seed, 11, 13)
    img, lab = blob_volume(shape, 300 + seed, [2, 5], [(4, 5, 5), (5, 6, 8)], [(3, 4, 4), (3, 3, 4)], 14.0)
    alpha = float(rng.choice([1.0, 0.8, 1.3]))
    with ref_import.reference_modules():
        import importlib

        ac = importlib.import_module("biomedisa.features.active_contour")
        ref_a = ac.activeContour(img.copy(), lab.astype(np.uint8), alpha, 1 + seed % 2, 2)
        ref_r = ac.activeContour(img.copy(), lab.astype(np.uint8), simple=True)
    assert np.array_equal(A.active_contour(img, lab.astype(np.uint8), alpha, 1 + seed % 2, 2), ref_a)
    assert np.array_equal(A.active_contour(img, lab.astype(np.uint8), simple=True), ref_r)
