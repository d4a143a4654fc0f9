"""The reference's default quadrature tables (read_quad_info, src/QuadInfo.cpp:13-60;
the 20 / 130 / 923-point files of include/TetrahedralSEM.h:144-147, copied into
tests/golden by make_quad_tables.py).

CPU: the tables parse as the reference reads them and integrate what their names
claim (the 2-D and 3-D rules every monomial of degree <= 26 to 1e-14; the 1-D rule,
printed with 9 digits, polynomials of degree <= 19 to 1e-8).
GPU: a space with the tabulated rule computes right-hand side, Neumann and
Dirichlet data, errors and the interpolant exactly as the oracle with the same rule.
"""
import os
from math import factorial

import numpy as np
import pytest

from tsemlib_gb300.tsem import read_quad_tables

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
N_QP = [20, 130, 923]
FILES = [os.path.join(GOLDEN, f) for f in ("quad_info_1d_p38.dat", "quad_2d_deg26_n130.dat", "quad_3d_deg26_n923.dat")]


def _rule():
    return read_quad_tables(N_QP, FILES)


def test_default_tables_parse_and_are_exact():
    r = _rule()
    assert r["x1"].shape == (20,) and r["b2"].shape == (130, 3) and r["x3"].shape == (923, 3)
    for w in (r["w1"], r["w2"], r["w3"]):
        assert abs(w.sum() - 1.0) <= 1e-8
    assert np.all((r["x1"] > 0) & (r["x1"] < 1))
    assert np.allclose(r["b2"].sum(axis=1), 1.0)
    x, w = r["x3"], r["w3"]
    for deg in range(27):
        for a in range(deg + 1):
            for b in range(deg + 1 - a):
                c = deg - a - b
                exact = 6.0 * factorial(a) * factorial(b) * factorial(c) / factorial(deg + 3)
                num = float((w * x[:, 0] ** a * x[:, 1] ** b * x[:, 2] ** c).sum())
                assert abs(num - exact) <= 1e-14 * max(exact, 1e-30) + 1e-17
    b2, w2 = r["b2"], r["w2"]
    for deg in range(27):
        for a in range(deg + 1):
            c = deg - a
            exact = 2.0 * factorial(a) * factorial(c) / factorial(deg + 2)
            assert abs(float((w2 * b2[:, 0] ** a * b2[:, 1] ** c).sum()) - exact) <= 1e-14 * exact
    for k in range(20):
        assert abs(float((r["w1"] * r["x1"] ** k).sum()) - 1.0 / (k + 1)) <= 1e-8 / (k + 1)


@pytest.mark.gpu
@pytest.mark.parametrize("p,shuffle", [(4, False), (6, True)])
def test_tabulated_rule_matches_oracle(p, shuffle):
    import oracle
    from tsemlib_gb300 import manufactured as mf
    from tsemlib_gb300 import mesh, tsem
    m = mesh.kuhn_cube(3, 0.1, 5)
    if shuffle:
        m = mesh.shuffle_local_order(m, 6)
    m = mesh.mark_box_boundary(m, [(0, 0.0), (0, 1.0)])
    T = tsem.TSEM(p, 4, m)
    T.read_quad_info(N_QP, FILES)
    assert T.n_q_point == N_QP
    S = oracle.Space(m, p, quad_q=4)
    S.set_quadrature(**_rule())
    assert np.array_equal(T.element_qpoints().shape, (m.nt, 923, 3))
    b = T.calc_rhs(mf.f_cfg1)
    bo = S.rhs(mf.f_cfg1)
    assert np.abs(b - bo).max() <= 1e-13 * np.abs(bo).max()
    T.impose_neumann(b, mf.neumann_cfg1, 2)
    S.neumann(bo, mf.neumann_cfg1, 2)
    assert np.abs(b - bo).max() <= 1e-13 * np.abs(bo).max()
    A = T.stiff_matrix.copy()
    Ao = S.assemble("stiff")
    T.impose_boundary_condition(A, b, mf.u_cfg1, True, 1)
    S.dirichlet(Ao, bo, mf.u_cfg1, True, 1)
    assert np.abs(b - bo).max() <= 1e-12 * np.abs(bo).max()
    c = T.calc_interpolation(mf.u_cfg1)
    co = S.interpolation(mf.u_cfg1)
    assert np.abs(c - co).max() <= 1e-12 * np.abs(co).max()
    x = np.zeros(T.n_dof_total)
    tsem.TSEMSolver().solve_PCG(A, x, b, tol=1e-13, flag_preconditioner=1)
    e = T.calc_errors(x, mf.u_cfg1, mf.grad_cfg1)
    eo = S.errors(x, mf.u_cfg1, mf.grad_cfg1)
    assert abs(e[0] - eo[0]) <= 1e-10 * eo[0] and abs(e[1] - eo[1]) <= 1e-10 * eo[1]
