"""The reference's default quadrature tables (read_quad_info, src/QuadInfo.cpp:13-60;
the 20 / 130 / 923-point files of include/TetrahedralSEM.h:144-147, copied into
tests/golden by make_quad_tables.py).

CPU: the tables parse as the reference reads them and integrate what their names
claim (the 2-D and 3-D rules every monomial of degree <= 26 to 1e-14; the 1-D rule,
printed with 9 digits, polynomials of degree <= 19 to 1e-8).
CPU: the collapsed rule of q points per direction, in the library and in the
oracle, equals the reference's construction (build_quad_info, src/QuadInfo.cpp:63-119)
from the reference's own 1-D Gauss-Legendre tables (qinfo_1d_order<q>, gathered into
tests/golden/qinfo_1d_orders.txt) for every q = 2..64.
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


def _qinfo_1d():
    rules, q = {}, None
    for line in open(os.path.join(GOLDEN, "qinfo_1d_orders.txt")):
        tok = line.split()
        if tok[0] == "order":
            q = int(tok[1]); rules[q] = []
        else:
            rules[q].append((float(tok[0]), float(tok[1])))
    return {q: np.array(v) for q, v in rules.items()}


QINFO = _qinfo_1d()


def _build_quad_info(tab):
    """src/QuadInfo.cpp:63-119 restated on the file's rule, in the file's order:
    x = (1 + t) / 2, then the collapsed 2-D and 3-D rules over (i1, i2[, i3])."""
    x = 0.5 * (1 + tab[:, 0])
    w = tab[:, 1]
    q = len(x)
    i1, i2 = np.meshgrid(np.arange(q), np.arange(q), indexing="ij")
    i1, i2 = i1.ravel(), i2.ravel()
    b2 = np.stack([x[i1] * (1 - x[i2]), x[i2], 1 - x[i1] * (1 - x[i2]) - x[i2]], axis=1)
    w2 = 2 * (1 - x[i2]) * w[i1] * w[i2]
    j1, j2, j3 = (a.ravel() for a in np.meshgrid(np.arange(q), np.arange(q), np.arange(q), indexing="ij"))
    x3 = np.stack([x[j1] * (1 - x[j2]) * (1 - x[j3]), x[j2] * (1 - x[j3]), x[j3]], axis=1)
    w3 = 6 * (1 - x[j2]) * (1 - x[j3]) ** 2 * w[j1] * w[j2] * w[j3]
    return x, w, b2, w2, x3, w3


def test_reference_1d_tables_cover_orders_2_to_64():
    assert sorted(QINFO) == list(range(2, 65))
    for q, tab in QINFO.items():
        assert tab.shape == (q, 2)
        assert abs(tab[:, 1].sum() - 1.0) <= 1e-14       # weights of unit measure


@pytest.mark.parametrize("q", [2, 3, 4, 5, 6, 7, 8, 10, 12, 16, 20, 24, 32, 48, 64])
def test_collapsed_rule_matches_reference_construction(q):
    import oracle
    from tsemlib_gb300 import mesh, tsem
    x, w, b2, w2, x3, w3 = _build_quad_info(QINFO[q])
    # the file lists the nodes as -t1, t1, -t2, ...; both implementations ascend in x
    perm = np.argsort(x, kind="stable")
    m = mesh.mark_box_boundary(mesh.kuhn_cube(1, 0.0, 1), [(0, 0.0), (0, 1.0)])
    S = oracle.Space(m, 4, quad_q=q)
    for r in (tsem.TSEM(4, q, m, lazy=True).quadrature(), S.quadrature()):
        assert np.abs(r["x1"] - x[perm]).max() <= 4e-16
        # the tables carry 16 significant digits, and a 3-D weight is a product of
        # five rounded factors: agreement to 1e-14 of the largest weight
        assert np.abs(r["w1"] - w[perm]).max() <= 4e-15 * w.max()
        p2 = (perm[:, None] * q + perm[None, :]).ravel()
        assert np.abs(r["b2"] - b2[p2]).max() <= 1e-15
        assert np.abs(r["w2"] - w2[p2]).max() <= 1e-14 * w2.max()
        p3 = ((perm[:, None, None] * q + perm[None, :, None]) * q + perm[None, None, :]).ravel()
        assert np.abs(r["x3"] - x3[p3]).max() <= 1e-15
        assert np.abs(r["w3"] - w3[p3]).max() <= 1e-14 * w3.max()
