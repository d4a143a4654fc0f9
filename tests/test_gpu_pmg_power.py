"""solve_PMG (src/TSEMSolver.cpp:1446-1536) and solve_InversePower
(src/TSEMSolver.cpp:2042-2068) on the GPU against the oracle."""
import numpy as np
import pytest

import oracle
from tsemlib_gb300 import manufactured as mf
from tsemlib_gb300 import mesh, tsem

pytestmark = pytest.mark.gpu


def _poisson(n=2, p=4):
    m = mesh.mark_box_boundary(mesh.kuhn_cube(n, 0.1, 1), [(0, 0.0), (0, 1.0)])
    T = tsem.TSEM(p, p + 2, m)
    A = T.stiff_matrix.copy()
    b = T.calc_rhs(mf.f_cfg1)
    T.impose_neumann(b, mf.neumann_cfg1, 2)
    T.impose_boundary_condition(A, b, mf.u_cfg1, True, 1)
    return T, A, b


def test_solve_pmg_matches_oracle_iteration():
    T, A, b = _poisson()
    sol = tsem.TSEMSolver()
    sol.init_PMG(A, 4, T.calc_sum_dof(), order_step=2, smoother="gs")
    x = np.zeros(T.n_dof_total)
    st = sol.solve_PMG(x, b, tol=1e-9, max_step=200, smooth_step=2)
    assert st["status"] == "OK", st
    rp, c, v = A.arrays()
    Ao = oracle.Csr.from_arrays(rp, c, v)
    P = oracle.PMG(Ao, 4, T.calc_sum_dof(), 2)
    xo = np.zeros(T.n_dof_total)
    it = 0
    while np.abs(Ao.matvec(xo) - b).sum() >= 1e-9 and it <= 200:
        xo = P.vcycle(b, xo, smooth=2)
        it += 1
    assert st["iterations"] == it
    assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()


def test_inverse_power_matches_oracle():
    m = mesh.mark_all_boundary(mesh.kuhn_cube(2, 0.0, 1))
    T = tsem.TSEM(4, 6, m)
    A = T.stiff_matrix.copy()
    B = T.mass_matrix.copy()
    T.impose_zero_boundary_condition(A, None, 1)
    T.impose_zero_boundary_condition(B, None, 1)
    x0 = np.random.default_rng(4).uniform(0.0, 1.0, T.n_dof_total)
    T.impose_zero_boundary_condition(None, x0, 1)
    x = x0.copy()
    sol = tsem.TSEMSolver()
    e = sol.solve_InversePower(x, A, B, tol=1e-12, max_step=1000)
    rp, c, v = A.arrays()
    Ao = oracle.Csr.from_arrays(rp, c, v)
    rp, c, v = B.arrays()
    Bo = oracle.Csr.from_arrays(rp, c, v)
    eo, xo, _ = oracle.inverse_power(Ao, Bo, x0, tol=1e-12, max_step=1000)
    assert e == pytest.approx(eo, rel=1e-10)
    assert abs(e - 3 * np.pi ** 2) / (3 * np.pi ** 2) < 1e-2
    assert np.abs(np.abs(x) - np.abs(xo)).max() <= 1e-6 * np.abs(xo).max()


@pytest.mark.parametrize("flag,omega,sweeps", [(3, 1.0, 1), (3, 1.5, 2)])
def test_ssor_preconditioner_matches_oracle(flag, omega, sweeps):
    """solve_PCG flag 3 (ite_SSOR, src/TSEMSolver.cpp:1307-1345) to convergence."""
    T, A, b = _poisson()
    sol = tsem.TSEMSolver()
    x = np.zeros(T.n_dof_total)
    st = sol.solve_PCG(A, x, b, tol=1e-9, max_step=2000, flag_preconditioner=flag, ite_step=sweeps, var=omega)
    assert st["status"] == "OK", st
    rp, c, v = A.arrays()
    Ao = oracle.Csr.from_arrays(rp, c, v)
    xo, so = oracle.pcg(Ao, b, tol=1e-9, max_step=2000, flag=flag, smooth=sweeps, omega=omega)
    assert st["iterations"] == so["iterations"]
    assert np.abs(x - xo).max() <= 1e-9 * np.abs(xo).max()


def test_sor_preconditioner_matches_oracle_iterates():
    """solve_PCG flag 2 (ite_SOR, src/TSEMSolver.cpp:1288-1304): a forward sweep is not a
    symmetric preconditioner and CG need not converge with it, so the test follows the
    first 15 iterations of both implementations."""
    T, A, b = _poisson()
    sol = tsem.TSEMSolver()
    x = np.zeros(T.n_dof_total)
    st = sol.solve_PCG(A, x, b, tol=1e-30, max_step=15, flag_preconditioner=2, ite_step=1, var=1.2)
    rp, c, v = A.arrays()
    Ao = oracle.Csr.from_arrays(rp, c, v)
    xo, so = oracle.pcg(Ao, b, tol=1e-30, max_step=15, flag=2, smooth=1, omega=1.2)
    assert st["iterations"] == so["iterations"]
    assert np.abs(x - xo).max() <= 1e-8 * np.abs(xo).max()
