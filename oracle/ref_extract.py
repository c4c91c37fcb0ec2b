"""Build recipe for oracle/_ref — the reference's OWN kernels compiled for the
CPU. Test infrastructure and CPU baseline only; outputs go to oracle/_ref/
(git-ignored) and nothing from the reference is committed.

Step 1 (needs the reference tree, i.e. this container): import the
reference's kernel factories with stubbed pycuda/pyopencl
(``ref_import.reference_modules``) and write the source strings they would
JIT-compile into ``_ref/ref_sources.inc``, each wrapped in renaming macros:
  * pycuda_small._build_kernel_int8/_float32           (walkers, CUDA small path)
  * pycuda_small_allx._build_kernel_int8/_float32      (walkers, CUDA all-axis)
  * pycuda_large_allx._build_kernel_int8/_float32      (walkers, CUDA all-axis large path: adaptive seeds)
  * pycuda_large._build_kernel_int8/_float32          (walkers, CUDA large path: adaptive seeds)
  * pyopencl_small._build_kernel('char'|'float','uchar') (walkers, OpenCL)
  * gpu_kernels._build_curvature_gpu/_build_update_gpu/_build_kernel_max/
    _build_kernel_uncertainty                            (post kernels)
Step 2 (anywhere, also on the GPU host from the copied .inc): compile
``ref_driver.c`` + the .inc with gcc into
  * ``_ref/libref_pin.so``  (-O2 -ffp-contract=off: binary32 ops round one by one)
  * ``_ref/libref_fast.so`` (-O3, compiler defaults: the timed CPU baseline).
Usage: ``python oracle/ref_extract.py``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF = HERE / "_ref"
INC = REF / "ref_sources.inc"
PIN = REF / "libref_pin.so"
FAST = REF / "libref_fast.so"

# (factory module, factory, args, renamed entry, entry name in the source)
_KERNELS = [
    ("biomedisa.features.random_walk.pycuda_small", "_build_kernel_int8", (), "ref_cuda_walk_i8", "Funktion"),
    ("biomedisa.features.random_walk.pycuda_small", "_build_kernel_float32", (), "ref_cuda_walk_f32", "Funktion"),
    ("biomedisa.features.random_walk.pycuda_large", "_build_kernel_int8", (), "ref_cuda_walk_large_i8", "Funktion"),
    ("biomedisa.features.random_walk.pycuda_large", "_build_kernel_float32", (), "ref_cuda_walk_large_f32",
     "Funktion"),
    ("biomedisa.features.random_walk.pycuda_small_allx", "_build_kernel_int8", (), "ref_cuda_walk_allx_i8",
     "Funktion"),
    ("biomedisa.features.random_walk.pycuda_small_allx", "_build_kernel_float32", (), "ref_cuda_walk_allx_f32",
     "Funktion"),
    ("biomedisa.features.random_walk.pycuda_large_allx", "_build_kernel_int8", (), "ref_cuda_walk_large_allx_i8",
     "Funktion"),
    ("biomedisa.features.random_walk.pycuda_large_allx", "_build_kernel_float32", (),
     "ref_cuda_walk_large_allx_f32", "Funktion"),
    ("biomedisa.features.random_walk.pyopencl_small", "_build_kernel", ("char", "uchar"), "ref_ocl_walk_char",
     "randomWalk"),
    ("biomedisa.features.random_walk.pyopencl_small", "_build_kernel", ("float", "uchar"), "ref_ocl_walk_float",
     "randomWalk"),
    ("biomedisa.features.random_walk.gpu_kernels", "_build_curvature_gpu", (), "ref_curvature", "Funktion"),
    ("biomedisa.features.random_walk.gpu_kernels", "_build_update_gpu", (), "ref_update", "Funktion"),
    ("biomedisa.features.random_walk.gpu_kernels", "_build_kernel_max", (), "ref_max", "Funktion"),
    ("biomedisa.features.random_walk.gpu_kernels", "_build_kernel_uncertainty", (), "ref_uncertainty",
     "Funktion"),
]


def extract() -> Path:
    """Writes _ref/ref_sources.inc from the reference tree."""
    import importlib

    sys.path.insert(0, str(HERE))
    from ref_import import REFERENCE_ROOT, capture, reference_modules

    if not Path(REFERENCE_ROOT).is_dir():
        raise FileNotFoundError(
            f"reference tree not found at {REFERENCE_ROOT}: set BIOMEDISA_REFERENCE_ROOT to the reference checkout")
    REF.mkdir(exist_ok=True)
    parts = ["/* generated by oracle/ref_extract.py from the reference tree; do not commit */\n"]
    with reference_modules():
        for mod, fn, args, new, old in _KERNELS:
            m = importlib.import_module(mod)
            src = capture(getattr(m, fn), *args)
            parts.append(f"#define {old} {new}\n#define _calc_var {new}__calc_var\n#define weight {new}__weight\n")
            parts.append(src)
            parts.append(f"\n#undef {old}\n#undef _calc_var\n#undef weight\n")
    tmp = INC.with_suffix(".tmp")
    tmp.write_text("".join(parts))
    os.replace(tmp, INC)
    return INC


def compile_libs() -> tuple[Path, Path]:
    if not INC.exists():
        raise FileNotFoundError(f"{INC} missing: run the extraction step where the reference tree exists")
    common = ["-fopenmp", "-fsigned-char", "-fPIC", "-shared", "-w", f"-I{HERE}", str(HERE / "ref_driver.c"), "-lm"]
    for out, opt in ((PIN, ["-O2", "-ffp-contract=off", "-fno-fast-math"]), (FAST, ["-O3"])):
        tmp = out.with_suffix(".so.tmp")
        subprocess.run(["gcc", *opt, *common, "-o", str(tmp)], check=True)
        os.replace(tmp, out)
    return PIN, FAST


def build(extract_if_possible: bool = True) -> bool:
    """Extracts (when the reference tree is present) and compiles. Returns
    False when neither the tree nor a previously extracted .inc exists."""
    sys.path.insert(0, str(HERE))
    from ref_import import REFERENCE_ROOT

    if extract_if_possible and Path(REFERENCE_ROOT).is_dir():
        extract()
    if not INC.exists():
        return False
    newest = max(INC.stat().st_mtime, (HERE / "ref_driver.c").stat().st_mtime, (HERE / "ref_shim.h").stat().st_mtime)
    if not (PIN.exists() and FAST.exists() and min(PIN.stat().st_mtime, FAST.stat().st_mtime) >= newest):
        compile_libs()
    return True


if __name__ == "__main__":
    sys.path.insert(0, str(HERE))
    ok = build()
    print("oracle/_ref built" if ok else "oracle/_ref unavailable (no reference tree and no extracted sources)")
