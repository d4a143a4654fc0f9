"""The multi-index numbering pinned to TSEMLib's own code (no GPU needed).

TSEMLib's Correspondence<3> (include/Correspondence.h:64-109) numbers the Jacobi
basis: every reference-element matrix, transform and DOF offset is indexed by it.
Its header compiles on its own, so tests/golden/multiindex_M12.txt is the output of
the reference's code itself (oracle/ref_correspondence.cpp built against the
reference tree by tests/golden/make_multiindex_table.py).  Both the oracle's table
and the library's (tsem_multiindex) must equal it exactly for orders 0..12, and the
per-degree ranges must equal the counts both sides use."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from tsemlib_gb300 import tsem

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "multiindex_M12.txt")
REF_EXE = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "ref_correspondence")


def _load(text):
    tables = {}
    cur = None
    for line in text.splitlines():
        tok = line.split()
        if tok[0] == "M":
            cur = {"n": int(tok[2]), "range": [], "num": []}
            tables[int(tok[1])] = cur
        elif tok[0] == "range":
            cur["range"].append([int(t) for t in tok[1:]])
        elif tok[0] == "num":
            cur["num"].append([int(t) for t in tok[1:]])
    return {M: {"n": t["n"], "range": np.array(t["range"]), "num": np.array(t["num"])} for M, t in tables.items()}


REF = _load(open(FIXTURE).read())


def test_fixture_covers_orders_0_to_12():
    assert sorted(REF) == list(range(13))
    for M, t in REF.items():
        assert t["n"] == (M + 1) * (M + 2) * (M + 3) // 6
        assert len(t["num"]) == t["n"]
        assert np.array_equal(t["num"][:, 0], np.arange(t["n"]))
        assert np.array_equal(t["num"][:, 4], np.arange(t["n"]))     # index2number(number2index(i)) = i


@pytest.mark.parametrize("M", range(13))
def test_library_and_oracle_number_like_the_reference(M):
    t = REF[M]
    alpha_ref = t["num"][:, 1:4]
    for alpha, number in (tsem.multiindex(M), oracle.multiindex(M)):
        assert np.array_equal(alpha, alpha_ref)
        assert np.array_equal(number, np.arange(t["n"]))
    # n_index_begin(order) / n_index_end(order): the numbers of degree < order and <= order
    deg = alpha_ref.sum(axis=1)
    for order, begin, end in t["range"]:
        assert begin == np.count_nonzero(deg < order) and end == np.count_nonzero(deg <= order)


def test_reference_build_reproduces_fixture():
    if not os.path.exists(REF_EXE):
        pytest.skip("oracle/_ref not built (needs the reference tree; `make -C oracle ref`)")
    out = subprocess.run([REF_EXE, "12"], check=True, capture_output=True, text=True).stdout
    assert out == open(FIXTURE).read()


def test_multiindex_rejects_orders_out_of_range():
    from tsemlib_gb300 import _lib
    L = _lib.lib()
    for M in (-1, 41):
        assert L.tsem_multiindex(M, None, None) == 6      # TSEM_INVALID
        msg = L.tsem_last_error()
        assert "order must be in [0, 40]" in (msg.decode() if isinstance(msg, bytes) else str(msg))
    assert L.tsem_multiindex(40, None, None) == 0


def test_cpp_correspondence_prints_the_reference_tables(tmp_path):
    """tsem_gpu::Correspondence (include/tsem_gpu.hpp), the C++ surface's stand-in for
    Correspondence<3>, printed in the reference driver's layout by
    tests/cpp/correspondence_dump.cpp, equals the reference code's output byte for
    byte (host only)."""
    from tests.cpp_shim import LIBDIR, build_shim
    if not os.path.exists(os.path.join(LIBDIR, "libtsemgpu.so")):
        pytest.skip("library not built")
    exe = build_shim(str(tmp_path), "correspondence_dump")
    out = subprocess.run([exe, "12"], check=True, capture_output=True, text=True).stdout
    assert out == open(FIXTURE).read()
