"""Imports modules of the reference (biomedisa) in this container — TEST
INFRASTRUCTURE ONLY, used by the oracle's extraction recipe and by the
golden-fixture generator; never imported by the product or on the GPU host.

The reference's third-party dependencies are missing here, so they are
replaced by stubs while importing:
  * ``pycuda.compiler.SourceModule`` and ``pyopencl.Program`` record the
    kernel source strings they are given (no compilation);
  * ``numba.jit`` returns the undecorated Python function;
  * every other missing module is an empty placeholder.
Nothing under the reference tree is written (bytecode writing is disabled).
"""
from __future__ import annotations

import importlib
import os
import sys
import types
from contextlib import contextmanager

# Where the reference checkout lives. This recipe reads the reference from
# there; set BIOMEDISA_REFERENCE_ROOT to use another checkout. Every other file
# takes the location from here.
REFERENCE_ROOT = os.environ.get("BIOMEDISA_REFERENCE_ROOT", "/root/reference")

RECORDED_SOURCES: list[str] = []


class _Anything(types.ModuleType):
    """Placeholder module: any attribute is another placeholder callable."""

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _AnyCallable()


class _AnyCallable:
    def __call__(self, *a, **k):
        return _AnyCallable()

    def __getattr__(self, name):
        return _AnyCallable()


class _SourceModule:
    def __init__(self, code, *a, **k):
        RECORDED_SOURCES.append(code)
        self.code = code

    def get_function(self, name):
        return _AnyCallable()


class _Program:
    def __init__(self, ctx, code):
        RECORDED_SOURCES.append(code)
        self.code = code

    def build(self, *a, **k):
        return _AnyCallable()


class _NumbaF32:
    """A float32 scalar read from a float32 array inside a numba-compiled
    function, with numba's typing of the operations geodesic_raster_scan
    (geodis.py:44-76) applies to it:
      float32 - float32  -> float32 (binary32 subtraction)
      float32 ** int     -> float32 (repeated binary32 multiplication, as
                            numba's integer power does)
      float32 + float64, float64 * float32 -> float64
      comparisons        -> on the exact values.
    Plain NumPy-2 scalars differ: a Python float added to an np.float32 stays
    float32 there (NEP 50), where numba computes in float64."""

    __slots__ = ("v",)

    def __init__(self, v):
        import numpy as np

        self.v = np.float32(v)

    def __sub__(self, o):
        return _NumbaF32(self.v - o.v)

    def __pow__(self, k):
        import numpy as np

        if not isinstance(k, int) or k < 0:
            raise TypeError("only non-negative integer powers are emulated")
        r, a = np.float32(1.0), self.v
        while True:
            if k & 1:
                r = np.float32(r * a)
            k >>= 1
            if not k:
                return _NumbaF32(r)
            a = np.float32(a * a)

    def __add__(self, o):
        return float(self.v) + float(o)

    __radd__ = __add__

    def __rmul__(self, o):
        return float(o) * float(self.v)

    def __float__(self):
        return float(self.v)

    def __lt__(self, o):
        return float(self.v) < float(o)

    def __gt__(self, o):
        return float(self.v) > float(o)


class _NumbaF32Array:
    """View of a float32 array whose reads give _NumbaF32 scalars and whose
    stores round a float64 value to float32, as numba's setitem does."""

    def __init__(self, a):
        self.a = a
        self.shape = a.shape

    def __getitem__(self, idx):
        return _NumbaF32(self.a[idx])

    def __setitem__(self, idx, value):
        import numpy as np

        self.a[idx] = np.float32(float(value))


def _numba_typed(f):
    """Runs a numba-compiled function as Python with numba's scalar typing
    where plain Python/NumPy-2 typing differs.
    smooth_img_3x3 (biomedisa_helper.py:308-323) starts its accumulator at the
    integer 0, which numba types as int64 (float64 once a float is added);
    under NumPy 2 rules a Python 0 plus a uint8 scalar stays uint8 and
    overflows. The input is widened to int64/float64 for the call and the
    result cast back to the input dtype, as numba's store into the
    uint8/float32 output does.
    geodesic_raster_scan (geodis.py:44-76) runs on float32 views that follow
    numba's float32/float64 typing (_NumbaF32).
    Active contour (curvop_numba.py, active_contour.py):
      * evolution (:5-29): numba types the Python float ``alpha`` as float64,
        so ``alpha * abs(float32)`` is a binary64 product; under NumPy 2 a
        Python float times an np.float32 stays float32. alpha is passed as an
        np.float64, which restores the binary64 product.
      * erosion / dilation (:31-84): numba computes ``start[...] - label`` and
        the running sum in int64; on uint8 NumPy scalars they wrap modulo 256
        (a plane sum of 256 would read as 0). The label volume is read through
        an int64 copy; the stores into the uint8 output are unchanged.
      * geodis (active_contour.py:45-81): the float32 map is read through a
        _NumbaF32Array (float32 + float64 and float32 + int64 are binary64 in
        numba, the minimum is stored rounded to float32)."""
    name = getattr(f, "__name__", "")
    if name == "evolution":

        def evolution(mean, A, data, alpha):
            import numpy as np

            return f(mean, A, data, np.float64(alpha))

        evolution.__name__ = name
        return evolution
    if name in ("erosion", "dilation"):

        def morph(start, final, P3, zsh, ysh, xsh, label):
            import numpy as np

            f(start.astype(np.int64), final, P3, zsh, ysh, xsh, int(label))
            return start, final

        morph.__name__ = name
        return morph
    if name == "geodis":

        def geodis(c, sqrt2, sqrt3, iterations):
            import numpy as np

            if c.dtype != np.float32:
                raise TypeError("the typed emulation covers a float32 map only")
            f(_NumbaF32Array(c), sqrt2, sqrt3, iterations)
            return c

        geodis.__name__ = name
        return geodis
    if name == "geodesic_raster_scan":

        def scan(img, c, lamb=1.0, iterations=4):
            import numpy as np

            if img.dtype != np.float32 or c.dtype != np.float32:
                raise TypeError("the typed emulation covers float32 img and c only")
            f(_NumbaF32Array(img), _NumbaF32Array(c), lamb, iterations)
            return c

        scan.__name__ = name
        return scan
    if name != "smooth_img_3x3":
        return f

    def wrapper(img):
        import numpy as np

        wide = img.astype(np.float64 if np.issubdtype(img.dtype, np.floating) else np.int64)
        return f(wide).astype(img.dtype)

    wrapper.__name__ = f.__name__
    return wrapper


def _numba_jit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return _numba_typed(args[0])
    return _numba_typed


def _stubs():
    mods = {}
    pycuda = _Anything("pycuda")
    compiler = types.ModuleType("pycuda.compiler")
    compiler.SourceModule = _SourceModule
    mods.update({
        "pycuda": pycuda, "pycuda.compiler": compiler, "pycuda.driver": _Anything("pycuda.driver"),
        "pycuda.gpuarray": _Anything("pycuda.gpuarray"),
    })
    pyopencl = _Anything("pyopencl")
    pyopencl.Program = _Program
    mods["pyopencl"] = pyopencl
    mods["pyopencl.array"] = _Anything("pyopencl.array")
    numba = types.ModuleType("numba")
    numba.jit = _numba_jit
    numba.njit = _numba_jit
    numba.prange = range
    mods["numba"] = numba
    for name in ("tifffile", "medpy", "medpy.io", "skimage", "SimpleITK", "PIL", "cv2", "mpi4py",
                 "importlib_metadata", "netCDF4", "h5py"):
        try:
            if name in ("PIL",):
                raise ImportError
            importlib.import_module(name)
        except Exception:
            mods[name] = _Anything(name)
    for name in ("biomedisa.features.amira_to_np.amira_helper", "biomedisa.features.nc_reader"):
        m = types.ModuleType(name)
        m.amira_to_np = m.np_to_amira = m.nc_to_np = m.np_to_nc = _AnyCallable()
        mods[name] = m
    return mods


@contextmanager
def reference_modules():
    """Context in which ``import biomedisa...`` resolves to the reference."""
    saved = {k: sys.modules.get(k) for k in list(sys.modules) if k == "biomedisa" or k.startswith("biomedisa.")}
    for k in saved:
        del sys.modules[k]
    stubs = _stubs()
    old = {k: sys.modules.get(k) for k in stubs}
    sys.modules.update(stubs)
    old_path = list(sys.path)
    old_dwb = sys.dont_write_bytecode
    sys.dont_write_bytecode = True
    sys.path.insert(0, REFERENCE_ROOT)
    try:
        yield
    finally:
        sys.path[:] = old_path
        sys.dont_write_bytecode = old_dwb
        for k, v in old.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
        for k in [k for k in sys.modules if k == "biomedisa" or k.startswith("biomedisa.")]:
            del sys.modules[k]
        for k, v in saved.items():
            if v is not None:
                sys.modules[k] = v


def capture(fn, *args):
    """Calls a reference kernel factory and returns the source it compiled."""
    RECORDED_SOURCES.clear()
    ret = fn(*args)
    if isinstance(ret, str) and not RECORDED_SOURCES:
        return ret  # factories that return the source instead of compiling it
    if len(RECORDED_SOURCES) != 1:
        raise RuntimeError(f"expected one kernel source, got {len(RECORDED_SOURCES)}")
    return RECORDED_SOURCES[0]
