"""Geodesic interpolation on CPU: the oracle against the reference's own
outputs (tests/golden/ref_geo.npz, made by make_golden_geo.py), the launch
plan of si_geo_scan (host code of libsmartinterp.so, no device work) against
the reference's raster order, and the kernel's arithmetic, emulated wavefront
by wavefront in NumPy, against the oracle. The GPU kernels themselves are
checked in test_gpu_geodesic.py."""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))

import geo_oracle as G  # noqa: E402

GOLD = ROOT / "tests" / "golden" / "ref_geo.npz"
FWD = np.array([(-1, -1, -1), (-1, -1, 0), (-1, -1, 1), (-1, 0, -1), (-1, 0, 0), (-1, 0, 1), (-1, 1, -1),
                (-1, 1, 0), (-1, 1, 1), (0, -1, -1), (0, -1, 0), (0, -1, 1), (0, 0, -1)])


def _names(d, prefix):
    return sorted({k[len(prefix):].rsplit("_", 1)[0] for k in d.files if k.startswith(prefix)})


def test_oracle_segment_matches_reference_fixtures():
    d = np.load(GOLD)
    names = _names(d, "seg_")
    assert len(names) >= 6
    for n in names:
        with np.errstate(invalid="ignore", divide="ignore"):
            got = G.geodesic_segment(d[f"seg_{n}_image"], d[f"seg_{n}_labels"])
        assert np.array_equal(got, d[f"seg_{n}_result"]), n


def test_oracle_scan_matches_reference_fixtures():
    d = np.load(GOLD)
    names = _names(d, "scan_")
    assert len(names) >= 4
    for n in names:
        lamb, it = d[f"scan_{n}_params"]
        got = G.raster_scan(d[f"scan_{n}_img"].copy(), d[f"scan_{n}_c"].copy(), float(lamb), int(it))
        assert np.array_equal(got.view(np.uint32), d[f"scan_{n}_out"].view(np.uint32)), n


def test_oracle_matches_reference_live():
    """The reference's own geodesic_segment and geodesic_raster_scan, run here
    on fresh inputs (numba's scalar typing emulated), against the oracle."""
    import ref_import

    if not (Path(ref_import.REFERENCE_ROOT) / "biomedisa" / "geodis.py").exists():
        pytest.skip("reference tree not present")

    rng = np.random.default_rng(21)
    img = rng.integers(0, 255, size=(6, 8, 7)).astype(np.uint8)
    lab = np.zeros(img.shape, np.int32)
    lab[0, 1:7, 1:6] = rng.integers(0, 3, size=(6, 5))
    lab[5, 2:5, 2:5] = 2
    c0 = np.where(rng.random(img.shape) < 0.1, 0.0, np.inf).astype(np.float32)
    f = (rng.random(img.shape) * 2).astype(np.float32)
    with ref_import.reference_modules():
        import importlib

        geo = importlib.import_module("biomedisa.geodis")
        ref_seg = geo.geodesic_segment(img.copy(), lab.copy())
        ref_scan = geo.geodesic_raster_scan(f.copy(), c0.copy(), 0.3, 2)
    assert np.array_equal(G.geodesic_segment(img, lab), ref_seg)
    assert np.array_equal(G.raster_scan(f.copy(), c0.copy(), 0.3, 2).view(np.uint32), ref_scan.view(np.uint32))


# --- launch plan (host code of the library) ---------------------------------

def _visit_order(shape, fwd):
    from biomedisa_gb300 import _native as nat

    Z, Y, X = shape
    t = np.empty(shape, np.int32)
    rc = nat.lib().si_geo_visit_order(Z, Y, X, int(fwd), t.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0, nat.lib().si_last_error()
    return t


SHAPES = [(1, 5, 5), (2, 3, 3), (2, 5, 6), (3, 3, 4), (4, 4, 3), (5, 7, 9), (6, 4, 11), (9, 12, 7), (2, 10, 3),
          (7, 3, 15), (11, 6, 5)]


@pytest.mark.parametrize("shape", SHAPES)
def test_visit_order_reproduces_raster_dependencies(shape):
    Z, Y, X = shape
    for fwd in (1, 0):
        t = _visit_order(shape, fwd)
        dom = np.zeros(shape, bool)
        if Z >= 2 and Y >= 3 and X >= 3:
            zs = slice(1, Z) if fwd else slice(0, Z - 1)
            dom[zs, 1:Y - 1, 1:X - 1] = True
        # every voxel of the pass's domain exactly once (duplicates are refused by the library), nothing else
        assert np.array_equal(t >= 0, dom), (shape, fwd)
        zz, yy, xx = np.nonzero(dom)
        assert np.array_equal(t[zz, yy, xx], xx + 2 * yy + 4 * zz)
        # each neighbour a voxel reads is finished before it when the sequential scan has updated it
        sign = 1 if fwd else -1
        for dz, dy, dx in FWD * sign:
            qz, qy, qx = zz + dz, yy + dy, xx + dx
            inside = dom[qz, qy, qx]
            tq, tp = t[qz, qy, qx][inside], t[zz, yy, xx][inside]
            assert np.all(tq < tp) if fwd else np.all(tq > tp), (shape, fwd, (dz, dy, dx))


def _tile_order(shape, fwd):
    from biomedisa_gb300 import _native as nat

    arrs = [np.empty(shape, np.int32) for _ in range(3)]
    rc = nat.lib().si_geo_tile_visit_order(*shape, int(fwd), *(a.ctypes.data_as(ctypes.c_void_p) for a in arrs))
    assert rc == 0, nat.lib().si_last_error()
    return arrs


TILE_SHAPES = SHAPES + [(40, 70, 90), (9, 130, 45), (70, 20, 33), (12, 12, 300)]


@pytest.mark.parametrize("shape", TILE_SHAPES)
def test_tile_order_reproduces_raster_dependencies(shape):
    """Tiled mode: every neighbour a voxel reads (when the pass updates it)
    is finished in an earlier launch, or earlier in the same tile; the
    library also checks that each shared-memory neighbour is the scan's."""
    Z, Y, X = shape
    for fwd in (1, 0):
        wave, tile, step = _tile_order(shape, fwd)
        dom = np.zeros(shape, bool)
        if Z >= 2 and Y >= 3 and X >= 3:
            zs = slice(1, Z) if fwd else slice(0, Z - 1)
            dom[zs, 1:Y - 1, 1:X - 1] = True
        assert np.array_equal(wave >= 0, dom), (shape, fwd)
        zz, yy, xx = np.nonzero(dom)
        sign = 1 if fwd else -1
        for dz, dy, dx in FWD * sign:
            qz, qy, qx = zz + dz, yy + dy, xx + dx
            inside = dom[qz, qy, qx]
            wq, wp = wave[qz, qy, qx][inside], wave[zz, yy, xx][inside]
            same = (wq == wp)
            assert np.all(wq <= wp), (shape, fwd, (dz, dy, dx))
            tq, tp = tile[qz, qy, qx][inside][same], tile[zz, yy, xx][inside][same]
            sq, sp = step[qz, qy, qx][inside][same], step[zz, yy, xx][inside][same]
            assert np.all(tq == tp) and np.all(sq < sp), (shape, fwd, (dz, dy, dx))


# --- kernel arithmetic emulated on the launch plan ---------------------------

def _emulate_scan(img, c, lamb, iterations):
    """Wavefront-by-wavefront NumPy emulation of geo_wave_kernel: binary32
    difference and square; lamb == 1 -> binary32 sums and minimum, else the
    float64 expression, both as the kernel evaluates them."""
    Z, Y, X = img.shape
    f_img, f_c = img.ravel(), c.reshape(-1, Z * Y * X)
    offs = FWD[:, 0] * Y * X + FWD[:, 1] * X + FWD[:, 2]
    d = np.sqrt((FWD != 0).sum(1).astype(np.float64))
    w = (1.0 - lamb) * d
    orders = [(_visit_order(img.shape, f).ravel(), f) for f in (1, 0)]
    for _ in range(iterations):
        for t_of, fwd in orders:
            ts = np.unique(t_of[t_of >= 0])
            for t in (ts if fwd else ts[::-1]):
                v = np.nonzero(t_of == t)[0]
                for cl in f_c:
                    if lamb == 1.0:
                        best = cl[v].copy()
                        for n in range(13):
                            q = v + offs[n] if fwd else v - offs[n]
                            diff = f_img[v] - f_img[q]
                            cost = cl[q] + diff * diff
                            best = np.where(cost < best, cost, best)
                        cl[v] = best
                    else:
                        best = cl[v].astype(np.float64)
                        for n in range(13):
                            q = v + offs[n] if fwd else v - offs[n]
                            diff = f_img[v] - f_img[q]
                            cost = (cl[q].astype(np.float64) + w[n]) + lamb * (diff * diff).astype(np.float64)
                            best = np.where(cost < best, cost, best)
                        cl[v] = best.astype(np.float32)
    return c


@pytest.mark.parametrize("lamb,iterations", [(1.0, 4), (1.0, 1), (0.5, 2), (0.0, 1), (1.3, 2)])
def test_emulated_kernel_equals_oracle(lamb, iterations):
    rng = np.random.default_rng(int(lamb * 10) + iterations)
    with np.errstate(over="ignore", invalid="ignore"):
        for shape in ((5, 7, 9), (4, 6, 3), (2, 5, 4)):
            img = rng.random(shape).astype(np.float32)
            img[rng.random(shape) < 0.05] = np.float32(1e-30)  # tiny values: sums that round
            img[0, 0, 0] = np.nan
            c = np.where(rng.random((3,) + shape) < 0.15, 0.0, np.inf).astype(np.float32)
            c[1] = np.where(c[1] == 0, 0.0, rng.random(shape) * 1e6).astype(np.float32)
            c[2, 1, 1, 1] = -0.0
            want = np.stack([G.raster_scan(img, c[k].copy(), lamb, iterations) for k in range(3)])
            got = _emulate_scan(img, c.copy(), lamb, iterations)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), shape


def test_plan_geo_labels():
    from biomedisa_gb300.geodis import plan_geo_labels

    hist = np.zeros(258, np.int64)
    hist[[0, 3, 7]] = 5
    hist[256] = 2  # negatives are ignored regions
    labels, lut = plan_geo_labels(hist)
    assert labels.tolist() == [0, 3, 7]
    assert lut[0] == 0 and lut[3] == 1 and lut[7] == 2 and (np.delete(lut, [0, 3, 7]) == -1).all()
    hist[257] = 1
    with pytest.raises(ValueError):
        plan_geo_labels(hist)


def test_labels_for_device_preserves_values():
    from biomedisa_gb300.geodis import _labels_for_device

    rng = np.random.default_rng(1)
    base = rng.integers(-5, 250, size=(4, 5, 6))
    for dt, want in ((np.uint8, np.uint8), (np.int16, np.int16), (np.int32, np.int32), (np.int8, np.int16),
                     (np.uint16, np.int32), (np.int64, np.int32), (np.uint32, np.int32), (bool, np.uint8)):
        lab = (base > 100) if dt is bool else base.astype(dt)
        out = _labels_for_device(lab)
        assert out.dtype == want and out.flags.c_contiguous, dt
        assert np.array_equal(out.astype(np.int64), lab.astype(np.int64)), dt
    with pytest.raises(TypeError):
        _labels_for_device(base.astype(np.float32))
    with pytest.raises(ValueError):
        _labels_for_device(np.full((2, 2, 2), 2 ** 40, np.int64))


@pytest.mark.parametrize("shape", [(5, 7, 9), (40, 70, 90), (2, 3, 3), (1, 5, 5), (12, 12, 300)])
def test_scan_launch_counts(shape):
    """si_geo_scan_launches (host only for these modes) against the plans:
    one launch per non-empty voxel wavefront, or per tile-wavefront."""
    from biomedisa_gb300 import _native as nat

    n = ctypes.c_longlong(0)
    L = nat.lib()
    waves = sum(len(np.unique(t[t >= 0])) for t in (_visit_order(shape, f) for f in (1, 0)))
    assert L.si_geo_scan_launches(*shape, 1.0, 3, 1, ctypes.byref(n)) == 0
    assert n.value == 3 * waves
    assert L.si_geo_scan_launches(*shape, 0.5, 2, 4, ctypes.byref(n)) == 0
    tile_waves = [int(_tile_order(shape, f)[0].max()) + 1 for f in (1, 0)]
    if waves == 0:
        assert n.value == 0
    else:
        assert n.value >= 2 * sum(tile_waves)
        assert n.value <= 2 * sum(tile_waves) + 2 * 2  # a pass may end with empty tile-wavefronts
    assert L.si_geo_scan_launches(*shape, 1.0, 1, 6, ctypes.byref(n)) != 0


def _emulate_tiled(img, c, lamb, iterations):
    """The tiled scan's data flow in NumPy, from the library's own launch plan:
    per launch (tile-wavefront) every CTA sees the maps as they stood when the
    launch began, with the voxels of the other tiles of that launch poisoned
    (-inf: they may be mid-update), updates its own tile plane by plane and
    writes it back. A result equal to the sequential scan shows that no CTA
    uses a value another CTA of its launch is producing."""
    Z, Y, X = img.shape
    f_img = img.ravel()
    offs = FWD[:, 0] * Y * X + FWD[:, 1] * X + FWD[:, 2]
    w = (1.0 - lamb) * np.sqrt((FWD != 0).sum(1).astype(np.float64))
    plans = [(tuple(a.ravel() for a in _tile_order(img.shape, f)), f) for f in (1, 0)]
    out = c.reshape(-1, Z * Y * X).copy()
    for _ in range(iterations):
        for (wave, tile, step), fwd in plans:
            for S in range(int(wave.max()) + 1 if (wave >= 0).any() else 0):
                in_launch = wave == S
                start = out.copy()
                for T in np.unique(tile[in_launch]):
                    own = in_launch & (tile == T)
                    box = start.copy()
                    box[:, in_launch & ~own] = -np.inf
                    for k in np.unique(step[own]):
                        v = np.nonzero(own & (step == k))[0]
                        for cl in box:
                            if lamb == 1.0:
                                best = cl[v].copy()
                                for n in range(13):
                                    q = v + offs[n] if fwd else v - offs[n]
                                    diff = f_img[v] - f_img[q]
                                    best = np.where(cl[q] + diff * diff < best, cl[q] + diff * diff, best)
                                cl[v] = best
                            else:
                                best = cl[v].astype(np.float64)
                                for n in range(13):
                                    q = v + offs[n] if fwd else v - offs[n]
                                    diff = f_img[v] - f_img[q]
                                    cost = (cl[q].astype(np.float64) + w[n]) + lamb * (diff * diff).astype(np.float64)
                                    best = np.where(cost < best, cost, best)
                                cl[v] = best.astype(np.float32)
                    out[:, own] = box[:, own]
    return out.reshape(c.shape)


@pytest.mark.parametrize("shape,lamb", [((40, 70, 90), 1.0), ((9, 130, 45), 1.0), ((70, 20, 33), 0.5)])
def test_emulated_tiled_scan_equals_oracle(shape, lamb):
    rng = np.random.default_rng(shape[0])
    img = rng.random(shape).astype(np.float32)
    c = np.where(rng.random((2,) + shape) < 0.01, 0.0, np.inf).astype(np.float32)
    with np.errstate(invalid="ignore"):
        got = _emulate_tiled(img, c, lamb, 1)
    want = np.stack([G.raster_scan(img, c[k].copy(), lamb, 1) for k in range(2)])
    assert np.isfinite(got).sum() > 0.5 * got.size
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
