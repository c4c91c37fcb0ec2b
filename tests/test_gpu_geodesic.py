"""Geodesic interpolation on the device (si_geo_* through
biomedisa_gb300.geodis) against the reference's own outputs
(tests/golden/ref_geo.npz) and the oracle: bit-exact label volumes and
distance maps."""
import numpy as np
import pytest
import torch

import geo_oracle as G
from biomedisa_gb300 import _native as nat
from biomedisa_gb300 import geodis as D
from biomedisa_gb300 import synthetic as S
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _names(d, prefix):
    return sorted({k[len(prefix):].rsplit("_", 1)[0] for k in d.files if k.startswith(prefix)})


def test_reference_fixtures(cuda):
    d = np.load(GOLDEN / "ref_geo.npz")
    for n in _names(d, "seg_"):
        got = D.geodesic_segment(d[f"seg_{n}_image"], d[f"seg_{n}_labels"])
        assert got.dtype == np.uint8
        assert np.array_equal(got, d[f"seg_{n}_result"]), n
    for n in _names(d, "scan_"):
        lamb, it = d[f"scan_{n}_params"]
        c = d[f"scan_{n}_c"].copy()
        out = D.geodesic_raster_scan(d[f"scan_{n}_img"], c, float(lamb), int(it))
        assert out is c
        assert np.array_equal(c.view(np.uint32), d[f"scan_{n}_out"].view(np.uint32)), n


@pytest.mark.parametrize("dtype", [np.uint8, np.int8, np.uint16, np.int16, np.int32, np.float32, np.float64])
def test_segment_against_oracle_dtypes(dtype, cuda):
    rng = np.random.default_rng(np.dtype(dtype).num)
    img, lab, _ = S.plain_volume(seed=np.dtype(dtype).num, shape=(22, 27, 31), z_every=5, semi=(4, 9))
    if dtype in (np.float32, np.float64):
        img = (img.astype(dtype) * 3.7 - 100.0 + rng.normal(size=img.shape)).astype(dtype)
    elif dtype == np.int8:
        img = (img.astype(np.int16) - 128).astype(np.int8)
    elif dtype != np.uint8:
        img = (img.astype(np.int64) * 97 - (3000 if np.issubdtype(dtype, np.signedinteger) else 0)).astype(dtype)
    lab[3, 2:6, 2:6] = -1  # ignored region
    got = D.geodesic_segment(img, lab)
    with np.errstate(invalid="ignore", divide="ignore"):
        want = G.geodesic_segment(img, lab)
    assert np.array_equal(got, want), dtype


@pytest.mark.parametrize("lab_dtype", [np.uint8, np.int8, np.int16, np.uint16, np.int32, np.int64])
def test_segment_label_dtypes_and_gaps(lab_dtype, cuda):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 255, size=(12, 17, 19)).astype(np.uint8)
    img[:, :, 9:] //= 3
    lab = np.zeros(img.shape, np.int64)
    lab[0, 1:10, 1:9] = 200
    lab[0, 1:10, 10:18] = 17
    lab[11, 3:12, 4:15] = 5
    if np.issubdtype(lab_dtype, np.signedinteger):
        lab[6, 5:8, 5:8] = -3
    lab = lab.astype(lab_dtype)
    assert np.array_equal(D.geodesic_segment(img, lab), G.geodesic_segment(img, lab))


def test_segment_edge_cases(cuda):
    # no label at all, only negative labels, only one label, constant and NaN images, thin volumes
    rng = np.random.default_rng(8)
    img = rng.integers(0, 255, size=(5, 6, 7)).astype(np.uint8)
    for lab in (np.zeros(img.shape, np.int32), np.full(img.shape, -1, np.int32), np.full(img.shape, 4, np.int32)):
        assert np.array_equal(D.geodesic_segment(img, lab), G.geodesic_segment(img, lab))
    lab = np.zeros(img.shape, np.int32)
    lab[0, 2:4, 2:5] = 1
    lab[4, 1:3, 1:3] = 2
    flt = rng.random(img.shape).astype(np.float32)
    flt[2, 3, 3] = np.nan
    for im in (np.full(img.shape, 9, np.uint8), flt, np.where(flt > 0.5, -np.inf, flt).astype(np.float32)):
        with np.errstate(invalid="ignore", divide="ignore"):
            want = G.geodesic_segment(im, lab)
        assert np.array_equal(D.geodesic_segment(im, lab), want)
    for shape in ((1, 6, 7), (2, 3, 3), (3, 2, 9), (4, 9, 2), (2, 6, 7)):
        im = rng.integers(0, 255, size=shape).astype(np.uint8)
        lb = np.zeros(shape, np.int32)
        lb[0] = rng.integers(0, 3, size=shape[1:])
        assert np.array_equal(D.geodesic_segment(im, lb), G.geodesic_segment(im, lb)), shape


def test_segment_rejects_unsupported_labels(cuda):
    img = np.zeros((4, 5, 6), np.uint8)
    lab = np.zeros(img.shape, np.int32)
    lab[0, 1, 1] = 300
    with pytest.raises(ValueError):
        D.geodesic_segment(img, lab)
    with pytest.raises(TypeError):
        D.geodesic_segment(img, lab.astype(np.float32))


@pytest.mark.parametrize("lamb,iterations", [(1.0, 4), (0.5, 2), (0.0, 1), (0.25, 3)])
def test_scan_against_oracle(lamb, iterations, cuda):
    rng = np.random.default_rng(int(lamb * 100) + iterations)
    img = rng.random((19, 23, 29)).astype(np.float32)
    img[rng.random(img.shape) < 0.02] = np.float32(3e-30)
    c = np.where(rng.random(img.shape) < 0.01, 0.0, np.inf).astype(np.float32)
    c[5:9, 5:9, 5:9] = (rng.random((4, 4, 4)) * 5).astype(np.float32)
    want = G.raster_scan(img, c.copy(), lamb, iterations)
    got = D.geodesic_raster_scan(img, c.copy(), lamb, iterations)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    d_img = torch.from_numpy(img).to(cuda)
    for mode in range(6):
        d_c = torch.from_numpy(c).to(cuda)
        D.scan_device(d_c, d_img, lamb, iterations, mode)
        assert np.array_equal(d_c.cpu().numpy().view(np.uint32), want.view(np.uint32)), mode


@pytest.mark.parametrize("mode", [0, 3, 5])
def test_scan_graph_replays(mode, cuda):
    """Repeated scans of the same buffers: auto mode launches directly, then
    captures, then replays its graph; graph mode captures on the first call.
    Every call must give the oracle's maps."""
    rng = np.random.default_rng(30 + mode)
    img = rng.random((21, 18, 24)).astype(np.float32)
    c0 = np.where(rng.random((2,) + img.shape) < 0.02, 0.0, np.inf).astype(np.float32)
    want = np.stack([G.raster_scan(img, c0[k].copy(), 1.0, 4) for k in range(2)])
    d_img = torch.from_numpy(img).to(cuda)
    d_c0 = torch.from_numpy(c0).to(cuda)
    buf = torch.empty_like(d_c0)
    for call in range(4):
        buf.copy_(d_c0)
        D.scan_device(buf, d_img, 1.0, 4, mode)
        assert np.array_equal(buf.cpu().numpy().view(np.uint32), want.view(np.uint32)), (mode, call)
    other = torch.from_numpy(rng.random(img.shape).astype(np.float32)).to(cuda)  # same shape, other image
    buf.copy_(d_c0)
    D.scan_device(buf, other, 1.0, 4, mode)
    want2 = np.stack([G.raster_scan(other.cpu().numpy(), c0[k].copy(), 1.0, 4) for k in range(2)])
    assert np.array_equal(buf.cpu().numpy().view(np.uint32), want2.view(np.uint32))


@pytest.mark.parametrize("mode", [1, 2, 3, 4, 5])
def test_all_labels_in_one_scan_equal_separate_scans(mode, cuda):
    """si_geo_scan over nol stacked maps equals nol single-map scans."""
    rng = np.random.default_rng(4)
    img = torch.from_numpy(rng.random((17, 21, 25)).astype(np.float32)).to(cuda)
    c = torch.from_numpy(np.where(rng.random((4, 17, 21, 25)) < 0.02, 0.0, np.inf).astype(np.float32)).to(cuda)
    sep = [D.scan_device(c[k].clone(), img, mode=mode) for k in range(4)]
    D.scan_device(c, img, mode=mode)
    for k in range(4):
        assert torch.equal(c[k], sep[k]), k


@pytest.mark.parametrize("shape,nol", [((40, 300, 500), 1), ((60, 200, 300), 2)])
def test_cluster_scan_with_wide_wavefronts(shape, nol, cuda):
    """Wavefronts of up to 9606 (40x300x500) and 8196 (60x200x300) voxels,
    wider than one round of the cluster's 8192 threads, and the wavefront mode
    on the same maps."""
    rng = np.random.default_rng(shape[0])
    img = rng.random(shape).astype(np.float32)
    c = np.where(rng.random((nol,) + shape) < 0.001, 0.0, np.inf).astype(np.float32)
    want = np.stack([G.raster_scan(img, c[k].copy(), 1.0, 1) for k in range(nol)])
    d_img = torch.from_numpy(img).to(cuda)
    for mode in (D.SCAN_WAVEFRONTS, D.SCAN_CLUSTER, D.SCAN_TILES):
        d_c = torch.from_numpy(c).to(cuda)
        D.scan_device(d_c, d_img, 1.0, 1, mode)
        assert np.array_equal(d_c.cpu().numpy().view(np.uint32), want.view(np.uint32)), mode


@pytest.mark.parametrize("shape", [(40, 70, 90), (9, 130, 45), (70, 20, 33), (12, 12, 300), (3, 3, 3), (2, 9, 40)])
def test_tiled_scan_shapes(shape, cuda):
    """The tiled scan on shapes with several tiles along every axis, thin
    volumes and a single interior voxel, lamb 1 and 0.6."""
    rng = np.random.default_rng(sum(shape))
    img = rng.random(shape).astype(np.float32)
    c = np.where(rng.random((2,) + shape) < 0.01, 0.0, np.inf).astype(np.float32)
    d_img = torch.from_numpy(img).to(cuda)
    for lamb, it in ((1.0, 2), (0.6, 1)):
        want = np.stack([G.raster_scan(img, c[k].copy(), lamb, it) for k in range(2)])
        d_c = torch.from_numpy(c).to(cuda)
        D.scan_device(d_c, d_img, lamb, it, D.SCAN_TILES)
        assert np.array_equal(d_c.cpu().numpy().view(np.uint32), want.view(np.uint32)), (shape, lamb)


def test_segment_plain_volume_against_oracle(cuda):
    """The plain workload's volume kind (ellipsoids in noise, labels on every
    10th z-slice) at 64^3."""
    img, lab, _ = S.plain_volume(seed=5, shape=(64, 64, 64), z_every=10, semi=(8, 22))
    got = D.geodesic_segment(img, lab)
    assert np.array_equal(got, G.geodesic_segment(img, lab))
    assert len(np.unique(got)) == 3


def test_entry_points_reject_bad_arguments(cuda):
    L = nat.lib()
    x = torch.zeros(8, dtype=torch.float32, device=cuda)
    assert L.si_geo_scan(None, None, 4, 4, 4, 1, 1.0, 1, 0, None) == 1
    assert L.si_geo_scan(x.data_ptr(), x.data_ptr(), 2, 2, 2, 1, 1.0, 1, 6, None) == 1  # no mode 6
    assert L.si_geo_select(None, 1, 8, None, None, None) == 1
    assert L.si_geo_masks(None, 0, 8, None, 1, None, None) == 1
    mm = torch.zeros(4, dtype=torch.int32, device=cuda)
    assert L.si_geo_normalize(x.data_ptr(), 0, 0, x.data_ptr(), mm.data_ptr(), None) == 1
    assert L.si_geo_normalize(x.data_ptr(), 17, 8, x.data_ptr(), mm.data_ptr(), None) == 1
