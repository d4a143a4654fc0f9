"""A Poisson solve written against the C++ call surface (tests/cpp/shim_poisson.cpp)
gives the same DOF values as the same solve through the Python mirror (up to the
last bits of the data functions, which C++ evaluates with libm and Python with numpy)."""
import numpy as np
import pytest

from tsemlib_gb300 import manufactured as mf
from tests.cpp_shim import build_shim
from tsemlib_gb300 import mesh, tsem

pytestmark = pytest.mark.gpu


def test_cpp_shim_matches_python(tmp_path):
    import subprocess
    m = mesh.mark_box_boundary(mesh.kuhn_cube(3, 0.1, 5), [(0, 0.0), (0, 1.0)])
    p = 4
    with open(tmp_path / "mesh.bin", "wb") as fh:
        np.array([m.nv, m.nt], np.int32).tofile(fh)
        np.ascontiguousarray(m.xyz, np.float64).tofile(fh)
        np.ascontiguousarray(m.tet_v, np.int32).tofile(fh)
        for marks in (m.mark_v, m.mark_e, m.mark_f):
            np.array([len(marks)], np.int32).tofile(fh)
            np.ascontiguousarray(marks, np.int32).tofile(fh)
    exe = build_shim(str(tmp_path))
    r = subprocess.run([exe, str(tmp_path / "mesh.bin"), str(p), str(tmp_path / "out.bin")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    raw = (tmp_path / "out.bin").read_bytes()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    x_cpp = np.frombuffer(raw[8:8 + 8 * n], np.float64)
    l2, h1 = np.frombuffer(raw[8 + 8 * n:24 + 8 * n], np.float64)

    T = tsem.TSEM(p, p + 2, m)
    A = T.stiff_matrix.copy()
    b = T.calc_rhs(mf.f_cfg1)
    T.impose_neumann(b, mf.neumann_cfg1, 2)
    T.impose_boundary_condition(A, b, mf.u_cfg1, True, 1)
    sol = tsem.TSEMSolver()
    sol.init_PMG(A, p, T.calc_sum_dof(), order_step=2, smoother="gs")
    x = np.zeros(T.n_dof_total)
    sol.solve_PCG(A, x, b, tol=0.0, max_step=1000, flag_preconditioner=4, var=2, tol_rel=1e-12)
    assert n == T.n_dof_total
    assert np.abs(x_cpp - x).max() <= 1e-12 * np.abs(x).max()
    l2p, h1p = T.calc_errors(x, mf.u_cfg1, mf.grad_cfg1)
    assert l2 == pytest.approx(l2p, rel=1e-8) and h1 == pytest.approx(h1p, rel=1e-8)
    assert l2 < 1e-3
