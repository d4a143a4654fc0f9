"""Build libtsemgpu.so in-tree with nvcc for sm_103a (GB300).

    python -m tsemlib_gb300.build          # incremental
    python -m tsemlib_gb300.build --force
    python -m tsemlib_gb300.build --check  # the checked build, tsemlib_gb300/_build/check/

Translation units compile in parallel; the output goes to tsemlib_gb300/_build/.
The checked build compiles the same sources with -DTSEM_CHECK: bounds checks on the
matrix-free gathers and scatters and the FP32 SpMVs that record a failure and skip
the access (TSEM_LIB_VARIANT=check loads it).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtsemgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["basis.cpp", "space.cpp", "capi.cpp", "assemble.cu", "solve.cu", "physics.cu", "mf.cu", "lobpcg.cu", "serve.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-fopenmp",
          "-I", INCLUDE, "-I", CSRC]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))] + \
           [os.path.join(INCLUDE, "tsem_gpu.h")]


def out_dir(variant: str | None = None) -> str:
    return OUT_DIR if not variant else os.path.join(OUT_DIR, variant)


def lib_path(variant: str | None = None) -> str:
    return os.path.join(out_dir(variant), "libtsemgpu.so")


def _compile(src: str, force: bool, verbose: bool, variant: str | None = None) -> str:
    obj = os.path.join(out_dir(variant), os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    newest = max(os.path.getmtime(p) for p in [path] + _deps())
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    extra = ["-DTSEM_CHECK"] if variant == "check" else []
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "cu"] + ARCH + COMMON + extra + ["-c", path, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr, file=sys.stderr)
    return obj


def build(force: bool = False, verbose: bool = False, variant: str | None = None) -> str:
    """variant None: the library; "check": the checked build (-DTSEM_CHECK)."""
    if variant not in (None, "check"):
        raise ValueError(f"unknown build variant {variant!r}")
    os.makedirs(out_dir(variant), exist_ok=True)
    lib = lib_path(variant)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose, variant), SOURCES))
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, variant="check" if "--check" in sys.argv else None))
