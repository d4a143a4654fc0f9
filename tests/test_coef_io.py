"""Coefficient files (read_coef / write_coef, src/Miscellaneous.cpp:35-127): round
trip, and order lifting geometry by geometry (host only)."""
from math import comb

import numpy as np

from tsemlib_gb300 import mesh, tsem


def _space(p):
    m = mesh.mark_box_boundary(mesh.kuhn_cube(2, 0.1, 1), [(0, 0.0), (0, 1.0)])
    return m, tsem.TSEM(p, p + 2, m, lazy=True)


def test_round_trip(tmp_path):
    _, T = _space(4)
    x = np.random.default_rng(0).standard_normal((2, T.n_dof_total))
    f = str(tmp_path / "c.txt")
    T.write_coef(list(x), f)
    with open(f) as fh:
        assert fh.readline().split() == ["4", str(T.n_dof_total)]
    y = T.read_coef(f, n_vectors=2)
    assert np.allclose(y, x, rtol=1e-13, atol=0)


def test_order_lifting(tmp_path):
    m, T4 = _space(4)
    T6 = tsem.TSEM(6, 8, m, lazy=True)
    x = np.random.default_rng(1).standard_normal(T4.n_dof_total)
    f = str(tmp_path / "c.txt")
    T4.write_coef(x, f)
    y = T6.read_coef(f)
    lg4, la4 = T4.numbering()
    lg6, la6 = T6.numbering()
    ng = T4.n_geometry
    nz = 0
    for d in range(4):
        k4 = comb(3, d)
        for loc in range(sum(ng[:d]), sum(ng[:d + 1])):
            a, b = la4[lg4[loc]], la6[lg6[loc]]
            assert np.allclose(y[b:b + k4], x[a:a + k4], rtol=1e-13, atol=0)  # 14 significant digits in the file
            nz += k4
    assert np.count_nonzero(y) == nz == T4.n_dof_total
