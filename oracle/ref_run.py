"""Runs the REFERENCE's own smart_interpolation (biomedisa/interpolation.py,
rw_small.py, pycuda_small*.py, gpu_kernels.py) in this container — TEST
INFRASTRUCTURE ONLY (golden-fixture generation and oracle pinning).

pycuda and mpi4py are replaced by fakes: device arrays are NumPy buffers and a
"compiled" CUDA kernel is the reference's own kernel source compiled as C
(oracle/_ref/libref_pin.so, built by ref_extract.py), launched with the grid
the reference passes. mpi4py is a single-rank communicator. Everything else —
pre-processing, dtype handling, padding, cropping, slice reading, the
per-label launch loop, smoothing, uncertainty, argmax and get_labels — is the
reference's Python code, unmodified.
"""
from __future__ import annotations

import ctypes
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

import ref_extract  # noqa: E402
from ref_import import reference_modules  # noqa: E402

_lib = None


def ref_lib(kind: str = "pin"):
    """ctypes handle of oracle/_ref/libref_{pin,fast}.so (built on demand)."""
    global _lib
    if kind == "fast":
        if not ref_extract.build(extract_if_possible=False) and not ref_extract.build():
            raise FileNotFoundError("oracle/_ref unavailable")
        return ctypes.CDLL(str(ref_extract.FAST))
    if _lib is None:
        if not ref_extract.build():
            raise FileNotFoundError("oracle/_ref unavailable")
        _lib = ctypes.CDLL(str(ref_extract.PIN))
    return _lib


class FakeArray:
    """A 'device' buffer: a private NumPy array."""

    def __init__(self, arr):
        self.a = np.ascontiguousarray(arr).copy()

    def get(self, queue=None):
        return self.a.copy()

    @property
    def ptr(self):
        return ctypes.c_void_p(self.a.ctypes.data)


def _arg(x):
    if isinstance(x, FakeArray):
        return x.ptr
    if isinstance(x, (np.integer, int)):
        return ctypes.c_int(int(x))
    raise TypeError(f"unsupported kernel argument {type(x)}")


class _Kernel:
    def __init__(self, code):
        self.code = code
        if "a[index] = 0;" in code and "Funktion(float *a, int xsh, int ysh)" in code:
            self.kind = "fill"
        elif "Funktion(int axis" in code:
            self.kind = "walk_large_allx" if "Adaptive random walks" in code else "walk_allx"
        elif "Funktion(int segment" in code:
            self.kind = "walk_large" if "Adaptive random walks" in code else "walk"
        elif "curvature[index] = (dxx" in code:
            self.kind = "curvature"
        elif "phi[index] += 0.01" in code:
            self.kind = "update"
        elif "max[2 * vol + index] = tmp" in code:
            self.kind = "max"
        elif "1 - (1 - tmp) * (1 - tmp1)" in code:
            self.kind = "uncertainty"
        else:
            raise RuntimeError("unknown reference kernel source")
        self.variant = 0 if "(char*)" in code else 1

    def __call__(self, *args, block=None, grid=None):
        assert tuple(block) == (32, 32, 1), block
        gx, gy, gz = (int(g) for g in grid)
        lib = ref_lib()
        if self.kind == "fill":
            args[0].a.fill(0)
            return
        c = [_arg(a) for a in args]
        if self.kind == "walk":
            lib.ref_launch_walk(self.variant, gx, gy, gz, *c)
        elif self.kind == "walk_allx":
            lib.ref_launch_walk_allx(self.variant, gx, gy, gz, *c)
        elif self.kind == "walk_large":
            lib.ref_launch_walk_large(self.variant, gx, gy, gz, *c)
        elif self.kind == "walk_large_allx":
            lib.ref_launch_walk_large_allx(self.variant, gx, gy, gz, *c)
        else:
            kind = {"curvature": 0, "update": 1, "max": 2, "uncertainty": 3}[self.kind]
            lib.ref_launch_post(kind, gx, gy, gz, *c)


class _SourceModule:
    def __init__(self, code, *a, **k):
        self.k = _Kernel(code)

    def get_function(self, name):
        return self.k


class _Ctx:
    def pop(self):
        pass


class _Device:
    def __init__(self, i):
        self.i = i

    def make_context(self):
        return _Ctx()

    @staticmethod
    def count():
        return 1


def _memcpy_dtoh(dst, src):
    dst[...] = src.a.view(dst.dtype).reshape(dst.shape)


def _memcpy_htod(dst, src):
    dst.a.view(np.uint8).reshape(-1)[...] = np.frombuffer(np.ascontiguousarray(src).tobytes(), np.uint8)


class _Comm:
    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def send(self, *a, **k):
        pass

    def Send(self, *a, **k):
        pass

    def Barrier(self):
        pass

    def Allreduce(self, send, recv, op=None):
        recv[0][...] = send[0]

    def Split(self, color, key):
        return _Comm()


def _fakes():
    pycuda = types.ModuleType("pycuda")
    drv = types.ModuleType("pycuda.driver")
    drv.init = lambda: None
    drv.Device = _Device
    drv.mem_alloc = lambda nbytes: FakeArray(np.zeros(int(nbytes), np.uint8))
    drv.memcpy_dtoh = _memcpy_dtoh
    drv.memcpy_htod = _memcpy_htod
    ga = types.ModuleType("pycuda.gpuarray")
    ga.to_gpu = FakeArray
    ga.zeros = lambda shape, dtype=np.float32: FakeArray(np.zeros(shape, dtype))
    comp = types.ModuleType("pycuda.compiler")
    comp.SourceModule = _SourceModule
    pycuda.driver, pycuda.gpuarray, pycuda.compiler = drv, ga, comp
    mpi = types.ModuleType("mpi4py")
    MPI = types.ModuleType("mpi4py.MPI")
    MPI.COMM_WORLD = _Comm()
    MPI.Comm = _Comm
    MPI.FLOAT = MPI.INT = MPI.BYTE = None
    MPI.SUM = MPI.MAX = None
    mpi.MPI = MPI
    return {"pycuda": pycuda, "pycuda.driver": drv, "pycuda.gpuarray": ga, "pycuda.compiler": comp, "mpi4py": mpi,
            "mpi4py.MPI": MPI}


def reference_smart_interpolation(data, labelData, force_large=False, **kwargs):
    """Calls the reference's smart_interpolation (CUDA path) and returns its
    result dict. force_large=True sends the volume down the reference's large
    path (rw_large.py, pycuda_large*.py) as a volume above its size threshold
    would go (interpolation.py:196): the label count that pre_processing
    reports is inflated after it returns, which only that test reads."""
    kwargs.setdefault("platform", "cuda_force")
    ref_lib()
    with reference_modules():
        saved = {k: sys.modules.get(k) for k in _fakes()}
        sys.modules.update(_fakes())
        try:
            import biomedisa.interpolation as interp
            from biomedisa.interpolation import smart_interpolation

            if force_large:
                original = interp.pre_processing

                def pre_processing(bm):
                    bm = original(bm)
                    if bm.success:
                        bm.nol = 10 ** 12
                    return bm

                interp.pre_processing = pre_processing
            return smart_interpolation(data, labelData, **kwargs)
        finally:
            for k, v in saved.items():
                if v is None:
                    sys.modules.pop(k, None)
                else:
                    sys.modules[k] = v


def reference_helpers():
    """Imports the reference's host helper functions (with stubs) and returns
    them in a namespace; call only inside reference_modules()."""
    from biomedisa.features import biomedisa_helper as h

    return h
