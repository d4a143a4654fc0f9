"""The checked build (tsemlib_gb300/build.py --check, compiled with -DTSEM_CHECK).

There the matrix-free operator's gathers and scatters and the mixed solver's FP32
SpMVs check every index they read from a table against the length of the vector it
addresses; a failure is recorded, its access skipped, and the solve fails with
TSEM_INVALID.  The test runs a solve through the checked library in a child process
(the library a process loads is fixed by TSEM_LIB_VARIANT), then divides every bound
by two with the test hook tsem_debug_bounds: valid indices now fail the check, which
exercises the error path while every access that still happens stays inside its
vector.  The next solve with the real bounds gives the first solve's answer.  The
product build reports that it has no checks."""
import ctypes
import os
import subprocess
import sys
import textwrap

import pytest

from tsemlib_gb300 import _lib

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import ctypes
    import numpy as np
    from tsemlib_gb300 import _lib, mesh, tsem
    from tsemlib_gb300 import manufactured as mf
    L = _lib.lib()
    code, idx, on = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32()
    _lib.check(L.tsem_debug_bounds(1, ctypes.byref(code), ctypes.byref(idx), ctypes.byref(on)))
    assert on.value == 1 and code.value == 0, (on.value, code.value)
    m = mesh.mark_box_boundary(mesh.kuhn_cube(3, 0.1, 2), [(0, 0.0), (0, 1.0)])
    T = tsem.TSEM(6, 8, m)
    A = T.stiff_matrix.copy()
    b = T.calc_rhs(mf.f_cfg1)
    T.impose_neumann(b, mf.neumann_cfg1, 2)
    T.impose_boundary_condition(A, b, mf.u_cfg1, True, 1)
    mx = tsem.MixedSolver(T, A, 1, order_step=2, tol_rel=1e-10)
    x0 = np.zeros(T.n_dof_total)
    assert mx.solve(x0, b)["status"] == "OK"
    _lib.check(L.tsem_debug_bounds(0, ctypes.byref(code), ctypes.byref(idx), None))
    assert code.value == 0, (code.value, idx.value)
    _lib.check(L.tsem_debug_bounds(2, None, None, None))
    try:
        x1 = np.zeros(T.n_dof_total)
        try:
            mx.solve(x1, b)
            raise SystemExit("the halved bounds were not reported")
        except tsem.TsemError as e:
            assert e.status == 6 and "bounds check" in str(e), e
        _lib.check(L.tsem_debug_bounds(1, ctypes.byref(code), ctypes.byref(idx), None))
        assert code.value > 0 and idx.value >= 0, (code.value, idx.value)
    finally:
        L.tsem_debug_bounds(1, None, None, None)
    x2 = np.zeros(T.n_dof_total)
    assert mx.solve(x2, b)["status"] == "OK"
    assert np.abs(x2 - x0).max() <= 1e-9 * np.abs(x0).max()
    print("checked build ok")
""")


def test_checked_build_reports_and_recovers():
    from tsemlib_gb300 import build
    build.build(variant="check")
    env = dict(os.environ, TSEM_LIB_VARIANT="check")
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and "checked build ok" in r.stdout, r.stdout[-3000:] + r.stderr[-3000:]


def test_product_build_has_no_checks():
    on = ctypes.c_int32(1)
    _lib.check(_lib.lib().tsem_debug_bounds(0, None, None, ctypes.byref(on)))
    assert on.value == 0
