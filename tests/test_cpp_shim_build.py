"""The C++ call surface (include/tsem_gpu.hpp) compiles and links against the library."""
import os

import pytest

from tests.cpp_shim import LIBDIR, build_shim


def test_shim_compiles_and_links(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libtsemgpu.so")):
        pytest.skip("library not built")
    exe = build_shim(str(tmp_path))
    assert os.path.exists(exe)


def test_headers_compile_as_c_and_cpp(tmp_path):
    """include/tsem_gpu.h is plain C (C99, for C and FFI callers); include/tsem_gpu.hpp
    is C++17 over it."""
    import subprocess
    from tests.cpp_shim import ROOT
    inc = os.path.join(ROOT, "include")
    for cmd in (["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-fsyntax-only", "-x", "c",
                 os.path.join(inc, "tsem_gpu.h")],
                ["g++", "-std=c++17", "-Wall", "-Wextra", "-fsyntax-only", "-x", "c++",
                 os.path.join(inc, "tsem_gpu.hpp")]):
        r = subprocess.run(cmd, capture_output=True, text=True, cwd=str(tmp_path))
        assert r.returncode == 0 and "warning" not in r.stderr, r.stderr
