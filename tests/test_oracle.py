"""Internal consistency of the oracle (CPU): its NumPy, pure-Python and C
restatements agree bit for bit, and its weight function meets its error bound."""
import ctypes

import numpy as np
import pytest

import oracle as O
from biomedisa_gb300.synthetic import plain_volume, sparse_labels


def test_philox_numpy_python_c_agree(c_oracle):
    rng = np.random.default_rng(0)
    ctr = rng.integers(0, 2**32, size=(512, 4), dtype=np.uint64).astype(np.uint32)
    ctr[0] = 0
    ctr[1] = 0xFFFFFFFF
    for k0, k1 in ((0, 0), (0xFFFFFFFF, 0xFFFFFFFF), (0xA4093822, 0x299F31D0)):
        a = np.stack(O.philox4x32_10(ctr[:, 0], ctr[:, 1], ctr[:, 2], ctr[:, 3], k0, k1), 1)
        b = np.array([O.philox_python(tuple(int(x) for x in c), (k0, k1)) for c in ctr], np.uint32)
        c = np.zeros_like(ctr)
        c_oracle.or_philox(ctr.ctypes.data, k0, k1, c.ctypes.data, len(ctr))
        assert np.array_equal(a, b) and np.array_equal(a, c)


# Philox4x32-10 known answers (Salmon et al., SC'11; the Random123 test
# vectors): (counter, key) -> output.
PHILOX_KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF), (0xFFFFFFFF, 0xFFFFFFFF),
     (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def test_philox_known_answers(c_oracle):
    for ctr, key, out in PHILOX_KAT:
        assert tuple(O.philox_python(ctr, key)) == out
        a = O.philox4x32_10(*(np.array([v], np.uint32) for v in ctr), *key)
        assert tuple(int(w[0]) for w in a) == out
        c_in = np.array([ctr], np.uint32)
        c_out = np.zeros_like(c_in)
        c_oracle.or_philox(c_in.ctypes.data, key[0], key[1], c_out.ctypes.data, 1)
        assert tuple(int(v) for v in c_out[0]) == out


def test_philox_uniformity():
    """u01 of a Philox stream: mean 1/2, variance 1/12, flat histogram."""
    n = 1 << 18
    w = O.philox4x32_10(np.arange(n), 7, 3, 0, 11, 13)
    u = np.concatenate([O.u01(x) for x in w]).astype(np.float64)
    assert abs(u.mean() - 0.5) < 3e-3
    assert abs(u.var() - 1 / 12) < 1e-3
    h, _ = np.histogram(u, 64, (0, 1))
    chi2 = ((h - h.mean()) ** 2 / h.mean()).sum()
    assert chi2 < 130  # 63 dof, p ~ 1e-6


def _libm_fmaf():
    libm = ctypes.CDLL("libm.so.6")
    libm.fmaf.restype = ctypes.c_float
    libm.fmaf.argtypes = [ctypes.c_float] * 3
    return libm.fmaf


def test_fmaf_emulation_is_correctly_rounded():
    fmaf = _libm_fmaf()
    rng = np.random.default_rng(1)
    n = 20000
    x = (rng.standard_normal(n) * np.exp(rng.uniform(-15, 15, n))).astype(np.float32)
    y = (rng.standard_normal(n) * np.exp(rng.uniform(-15, 15, n))).astype(np.float32)
    z = (-(x.astype(np.float64) * y) * (1 + rng.standard_normal(n) * 1e-7)).astype(np.float32)
    z[::3] = rng.standard_normal(len(z[::3])).astype(np.float32)
    em = O.fmaf(x, y, z)
    ref = np.array([fmaf(float(a), float(b), float(c)) for a, b, c in zip(x, y, z)], np.float32)
    assert np.array_equal(em.view(np.uint32), ref.view(np.uint32))


def test_weight_numpy_equals_c(c_oracle):
    rng = np.random.default_rng(2)
    d2 = np.concatenate([rng.integers(0, 65026, 4000), np.arange(0, 300)]).astype(np.float32)
    c = O.weight_constant(rng.uniform(1, 5000, len(d2)).astype(np.float32))
    wn = O.edge_weight(d2, c)
    wc = np.array([c_oracle.or_weight_exp2(float(a), float(b)) for a, b in zip(d2, c)], np.float32)
    assert np.array_equal(wn.view(np.uint32), wc.view(np.uint32))
    cc = np.array([c_oracle.or_weight_constant(float(v)) for v in [1.0, 2.5, 77.25, 1e4]], np.float32)
    assert np.array_equal(cc, O.weight_constant(np.array([1.0, 2.5, 77.25, 1e4], np.float32)))


def test_weight_error_bound():
    """|w - 2^-y| <= 4e-7 * 2^-y for the rounded exponent y = RN(d2 c), and the
    flush to 0 only below 2^-125."""
    rng = np.random.default_rng(3)
    d2 = rng.uniform(0, 65025, 200000).astype(np.float32)
    c = rng.uniform(1e-5, 1.0, 200000).astype(np.float32)
    w = O.edge_weight(d2, c).astype(np.float64)
    y = (d2 * c).astype(np.float32).astype(np.float64)
    ex = np.exp2(-y)
    keep = y < 125
    assert np.all(np.abs(w[keep] - ex[keep]) <= 4e-7 * ex[keep])
    assert np.all(w[~keep] == 0)
    assert O.edge_weight(np.float32(0), np.float32(0.5)) == 1.0


def _case(seed, dtype, allaxis):
    img, lab, truth = plain_volume(seed=seed, shape=(30, 28, 26), z_every=4, semi=(5, 10))
    if allaxis:
        lab = sparse_labels(truth.astype(np.int32), z_every=5, y_every=6, x_every=6)
    if dtype == "f32":
        img = O.normalize_image(img.astype(np.uint16) * 3)
    data = np.pad(img, 1)
    l2 = np.pad(lab, 1)
    _, all_labels = O.pre_processing(l2)
    if allaxis:
        sl = [(0, k) for k, _ in O.read_indices_allx(l2, 0)]
        t1 = np.ascontiguousarray(np.swapaxes(l2, 0, 1))
        sl += [(1, k) for k, _ in O.read_indices_allx(t1, 1)]
        t2 = np.ascontiguousarray(np.swapaxes(t1, 0, 2))
        sl += [(2, k) for k, _ in O.read_indices_allx(t2, 2)]
    else:
        sl = [(0, k) for k in O.read_labeled_slices(l2)[0]]
    return data, l2, sl, all_labels


@pytest.mark.parametrize("dtype", ["u8", "f32"])
@pytest.mark.parametrize("allaxis", [False, True])
def test_walk_numpy_equals_c(dtype, allaxis):
    data, l2, sl, all_labels = _case(3, dtype, allaxis)
    seeds = O.extract_seeds(data, l2, sl, all_labels)
    assert len(seeds) > 100
    hn = O.walk_numpy(data, seeds, 2, 30, 12345, len(all_labels))
    hc = O.walk_c(data, seeds, 2, 30, 12345, len(all_labels))
    assert np.array_equal(hn, hc)
    assert hn.sum() > 0


def test_walk_c_thread_count_invariance():
    data, l2, sl, all_labels = _case(4, "u8", False)
    seeds = O.extract_seeds(data, l2, sl, all_labels)
    a = O.walk_c(data, seeds, 3, 50, 1, len(all_labels), nthreads=1)
    b = O.walk_c(data, seeds, 3, 50, 1, len(all_labels), nthreads=4)
    assert np.array_equal(a, b)


def test_walk_hits_bounded_and_interior():
    data, l2, sl, all_labels = _case(5, "u8", False)
    seeds = O.extract_seeds(data, l2, sl, all_labels)
    h = O.walk_c(data, seeds, 2, 40, 9, len(all_labels))
    assert h.sum() <= len(seeds) * 2 * 40
    assert h[:, 0].sum() == h[:, -1].sum() == h[:, :, 0].sum() == h[:, :, :, -1].sum() == 0


def test_smooth_f32_matches_scalar_restatement():
    """The vectorised smoothing step equals a scalar transcription of the
    reference curvature kernel (gpu_kernels.py:141-183) in binary32."""
    rng = np.random.default_rng(6)
    phi = rng.integers(0, 50, (6, 7, 8)).astype(np.float32)
    out = O.smooth_step(phi)
    f = np.float32
    exp = phi.copy()
    for z in range(1, 5):
        for y in range(1, 6):
            for x in range(1, 7):
                p = phi
                c = p[z, y, x]
                dx = f(f(p[z, y, x - 1] - p[z, y, x + 1]) * f(0.5))
                dxx = f(f(p[z, y, x - 1] - f(2 * c)) + p[z, y, x + 1])
                dy = f(f(p[z, y - 1, x] - p[z, y + 1, x]) * f(0.5))
                dyy = f(f(p[z, y - 1, x] - f(2 * c)) + p[z, y + 1, x])
                dz = f(f(p[z - 1, y, x] - p[z + 1, y, x]) * f(0.5))
                dzz = f(f(p[z - 1, y, x] - f(2 * c)) + p[z + 1, y, x])
                dx2, dy2, dz2 = f(dx * dx), f(dy * dy), f(dz * dz)
                dxy = f(f(f(f(p[z, y - 1, x - 1] + p[z, y + 1, x + 1]) - p[z, y - 1, x + 1]) - p[z, y + 1, x - 1])
                        * f(0.25))
                dxz = f(f(f(f(p[z + 1, y, x - 1] + p[z - 1, y, x + 1]) - p[z + 1, y, x + 1]) - p[z - 1, y, x - 1])
                        * f(0.25))
                dyz = f(f(f(f(p[z + 1, y - 1, x] + p[z - 1, y + 1, x]) - p[z + 1, y + 1, x]) - p[z - 1, y - 1, x])
                        * f(0.25))
                num = f(f(dxx * f(dy2 + dz2)) + f(dyy * f(dx2 + dz2)))
                num = f(num + f(dzz * f(dx2 + dy2)))
                num = f(num - f(f(f(2 * dx) * dy) * dxy))
                num = f(num - f(f(f(2 * dx) * dz) * dxz))
                num = f(num - f(f(f(2 * dy) * dz) * dyz))
                den = f(f(f(dx2 + dy2) + dz2) + f(1e-10))
                exp[z, y, x] = f(c + f(f(0.01) * f(num / den)))
    assert np.array_equal(out.view(np.uint32), exp.view(np.uint32))


def test_float_constants_match_cuda_literals():
    """The binary32 constants the kernels write as literals (0.01f, 1e-10f)
    equal numpy's float32 conversions used by the oracle."""
    import struct

    assert struct.unpack("<I", struct.pack("<f", 0.01))[0] == np.float32(0.01).view(np.uint32)
    assert struct.unpack("<I", struct.pack("<f", 1e-10))[0] == np.float32(1e-10).view(np.uint32)
    assert np.float32(0.01).view(np.uint32) == 0x3C23D70A
    assert np.float32(1e-10).view(np.uint32) == 0x2EDBE6FF
