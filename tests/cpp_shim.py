"""Helpers of the C++ shim tests: build tests/cpp/shim_poisson against the library."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "tsemlib_gb300", "_build")


def build_shim(out_dir):
    exe = os.path.join(out_dir, "shim_poisson")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "shim_poisson.cpp"), "-L", LIBDIR, "-ltsemgpu",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe
