"""Helpers of the C++ shim tests: build the programs of tests/cpp against the library."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "tsemlib_gb300", "_build")


def build_shim(out_dir, name="shim_poisson"):
    """Compile tests/cpp/<name>.cpp against include/ and link the library."""
    exe = os.path.join(out_dir, name)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-L", LIBDIR, "-ltsemgpu",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe
