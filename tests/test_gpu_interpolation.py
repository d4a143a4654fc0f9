"""calc_interpolation (src/Interpolation.cpp:104-216): exact for polynomials of the
space's degree, equal to the Dirichlet projection on boundary DOFs, and convergent."""
import numpy as np
import pytest

from tsemlib_gb300 import manufactured as mf
from tsemlib_gb300 import mesh, tsem

pytestmark = pytest.mark.gpu


def poly4(p):
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    return x * x * y - 0.5 * z ** 4 + x * y * z + 0.3 * y * y * z * x - 2.0 * x + 1.0


@pytest.mark.parametrize("shuffle", [False, True])
def test_polynomials_of_the_degree_are_reproduced(shuffle):
    m = mesh.kuhn_cube(2, 0.1, 6)
    if shuffle:
        m = mesh.shuffle_local_order(m, 7)
    m = mesh.mark_all_boundary(m)
    T = tsem.TSEM(4, 6, m)
    c = T.calc_interpolation(poly4)
    u = T.value_qp(c)
    ref = poly4(T.element_qpoints())
    assert np.abs(u - ref).max() <= 1e-11 * np.abs(ref).max()


def test_boundary_values_equal_the_dirichlet_projection():
    m = mesh.mark_box_boundary(mesh.kuhn_cube(2, 0.1, 1), [(0, 0.0), (0, 1.0)])
    T = tsem.TSEM(5, 7, m)
    c = T.calc_interpolation(mf.u_cfg1)
    A = T.stiff_matrix.copy()
    b = np.zeros(T.n_dof_total)
    T.impose_boundary_condition(A, b, mf.u_cfg1, True, 1)
    probe = np.ones(T.n_dof_total)
    T.impose_zero_boundary_condition(None, probe, 1)
    bnd = probe == 0
    d = np.array([A.arrays()[2][A.arrays()[0][i]] for i in np.nonzero(bnd)[0]])
    assert np.allclose(c[bnd], b[bnd] / d, rtol=1e-12, atol=1e-14)


def test_interpolation_error_decreases_with_order():
    m = mesh.mark_all_boundary(mesh.kuhn_cube(2, 0.1, 1))
    errs = []
    for p in (3, 5, 7):
        T = tsem.TSEM(p, p + 2, m)
        c = T.calc_interpolation(mf.u_cfg1)
        errs.append(T.calc_errors(c, mf.u_cfg1, mf.grad_cfg1)[0])
    assert errs[0] > 10 * errs[1] > 100 * errs[2]


@pytest.mark.parametrize("n,p,shuffle", [(2, 5, True), (6, 4, False)])
def test_interpolation_matches_oracle(n, p, shuffle):
    """The GPU interpolant equals the oracle's restatement of calc_interpolation
    (src/Interpolation.cpp:12-101) on every DOF: vertex, edge, face and interior."""
    import oracle
    m = mesh.kuhn_cube(n, 0.1, 3)
    if shuffle:
        m = mesh.shuffle_local_order(m, 4)
    m = mesh.mark_box_boundary(m, [(0, 0.0), (0, 1.0)])
    T = tsem.TSEM(p, p + 2, m)
    S = oracle.Space(m, p, quad_q=p + 2)
    c = T.calc_interpolation(mf.u_cfg1)
    c_o = S.interpolation(mf.u_cfg1)
    assert np.abs(c - c_o).max() <= 1e-12 * np.abs(c_o).max()
