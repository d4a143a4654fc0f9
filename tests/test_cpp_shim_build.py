"""The C++ call surface (include/tsem_gpu.hpp) compiles and links against the library."""
import os

import pytest

from tests.cpp_shim import LIBDIR, build_shim


def test_shim_compiles_and_links(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libtsemgpu.so")):
        pytest.skip("library not built")
    exe = build_shim(str(tmp_path))
    assert os.path.exists(exe)
