"""Order lifting by read_coef keeps the FE function: the hierarchical modes of order
p come first in every geometry block of order p' > p."""
import numpy as np
import pytest

from tsemlib_gb300 import mesh, tsem

pytestmark = pytest.mark.gpu


def test_lifted_function_is_unchanged(tmp_path):
    m = mesh.mark_box_boundary(mesh.kuhn_cube(2, 0.1, 1), [(0, 0.0), (0, 1.0)])
    T4 = tsem.TSEM(4, 8, m)
    T6 = tsem.TSEM(6, 8, m)
    x = np.random.default_rng(2).standard_normal(T4.n_dof_total)
    f = str(tmp_path / "c.txt")
    T4.write_coef(x, f)
    y = T6.read_coef(f)
    u4 = T4.value_qp(x)
    u6 = T6.value_qp(y)
    assert np.abs(u4 - u6).max() <= 1e-11 * np.abs(u4).max()
