"""The C-ABI library loads and exports every entry point the header declares
(no compute calls: this runs without a GPU)."""
import re

from conftest import ROOT


def declared_symbols():
    text = (ROOT / "include" / "smartinterp.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(si_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("si_walk", "si_extract_seeds", "si_argmax", "si_smooth", "si_label_histogram", "si_slice_flags"):
        assert s in syms


def test_library_exports_every_declared_symbol(native_lib):
    for s in declared_symbols():
        assert hasattr(native_lib, s), s


def test_python_binding_covers_header(native_lib):
    from biomedisa_gb300 import _native

    assert set(declared_symbols()) == set(_native.EXPORTED)


def test_version_and_error_state(native_lib):
    assert native_lib.si_version() >= 100
    assert native_lib.si_last_error() == b""


def test_argument_errors_without_launch(native_lib):
    """Null pointers are rejected before any CUDA call."""
    from biomedisa_gb300 import _native

    rc = native_lib.si_walk(None, 0, 8, 8, 8, None, None, 0, 1, 1, 0, None, 1, 0, 0, 0, None)
    assert rc == 1
    assert b"null pointer" in native_lib.si_last_error()
    rc = native_lib.si_smooth(None, None, None, 1, 4, 4, 4, 1, 0, None)
    assert rc == 1
    assert _native.SI_F32 == 5


def test_conv16_tc_argument_errors_without_launch(native_lib):
    """The tensor-core convolution rejects a bad stream count, dilation or
    shape before any CUDA call."""
    import ctypes

    assert native_lib.si_nn_conv16_tc_set_streams(3) == 1
    assert b"1, 2 or 4" in native_lib.si_last_error()
    assert native_lib.si_nn_conv16_tc_set_streams(1) == 0
    p = [ctypes.c_void_p(16 * (i + 1)) for i in range(4)]  # aligned, never dereferenced
    for dil in (0, 9):
        rc = native_lib.si_nn_conv16_tc(p[0], p[1], None, p[2], p[3], 1, 4, 4, 4, dil, 0, 0, None)
        assert rc == 1 and b"dilation" in native_lib.si_last_error()
    rc = native_lib.si_nn_conv16_tc(p[0], p[1], None, p[2], p[3], 0, 4, 4, 4, 1, 0, 0, None)
    assert rc == 1 and b"bad shape" in native_lib.si_last_error()
    rc = native_lib.si_nn_conv16_tc(ctypes.c_void_p(8), p[1], None, None, p[3], 1, 4, 4, 4, 1, 0, 0, None)
    assert rc == 1 and b"16-byte aligned" in native_lib.si_last_error()


def declared_arities():
    """Parameter count of every si_* declaration in the header."""
    text = (ROOT / "include" / "smartinterp.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(si_\w+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_binding_arities_match_header():
    """Every ctypes argument list has as many entries as the header's
    declaration has parameters (a drifted signature would pass garbage)."""
    from biomedisa_gb300 import _native

    ar = declared_arities()
    assert set(_native._SIGNATURES) <= set(ar)
    for name, args in _native._SIGNATURES.items():
        assert len(args) == ar[name], (name, len(args), ar[name])


def test_missing_library_fails_loudly(tmp_path):
    """Without libsmartinterp.so the binding raises: there is no CPU fallback."""
    import pytest

    from biomedisa_gb300 import _native

    with pytest.raises(ImportError, match="no CPU fallback"):
        _native.load(tmp_path / "libsmartinterp.so")


def test_entry_points_need_a_device_without_cuda():
    """On a host without a CUDA device the public calls raise instead of
    computing on the CPU."""
    import numpy as np
    import pytest
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from biomedisa_gb300 import geodis, smart_interpolation
    from biomedisa_gb300.active_contour import activeContour

    img = np.zeros((4, 5, 6), np.uint8)
    lab = np.zeros(img.shape, np.int32)
    lab[1, 1:3, 1:3] = 1
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        smart_interpolation(img, lab)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        activeContour(img, lab)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        geodis.geodesic_segment(img, lab)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        geodis.geodesic_raster_scan(img.astype(np.float32), np.zeros(img.shape, np.float32))


def test_device_tensor_apis_refuse_host_tensors():
    """Entry points that take device tensors refuse host tensors before any
    kernel could be handed a host pointer."""
    import pytest
    import torch

    from biomedisa_gb300 import geodis, interpolation, postprocess

    lab8 = torch.zeros((4, 5, 6), dtype=torch.uint8)
    for fn in (postprocess.clean, postprocess.fill):
        with pytest.raises(ValueError, match="CUDA"):
            fn(lab8, 0.5)
    img = torch.zeros((4, 5, 6), dtype=torch.uint8)
    lab = torch.zeros((4, 5, 6), dtype=torch.int32)
    with pytest.raises(ValueError, match="CUDA"):
        interpolation.DeviceJob(img, 0, lab, 4)
    with pytest.raises(ValueError, match="CUDA"):
        geodis.geodesic_segment_device(img, 0, lab, 4)
