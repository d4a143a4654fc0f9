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


def test_reading_a_higher_order_file_keeps_the_low_degree_modes(tmp_path):
    """A file of order 6 read into a space of order 4 keeps, geometry by geometry,
    the first modes of each block: the modes of degree <= 4 (edge, face and interior
    modes are ordered by degree).  The reference's loop copies all the file's modes
    of a geometry (src/Miscellaneous.cpp:57-64) and so writes past the block; here
    the block is cut to the space's order.  Writing the result back and lifting it
    to order 6 again returns the low-degree part of the original."""
    m, T4 = _space(4)
    T6 = tsem.TSEM(6, 8, m, lazy=True)
    x6 = np.random.default_rng(2).standard_normal(T6.n_dof_total)
    f6, f4 = str(tmp_path / "c6.txt"), str(tmp_path / "c4.txt")
    T6.write_coef(x6, f6)
    y4 = T4.read_coef(f6)
    lg4, la4 = T4.numbering()
    lg6, la6 = T6.numbering()
    ng = T4.n_geometry
    for d in range(4):
        k4 = comb(3, d)
        for loc in range(sum(ng[:d]), sum(ng[:d + 1])):
            a, b = la4[lg4[loc]], la6[lg6[loc]]
            assert np.allclose(y4[a:a + k4], x6[b:b + k4], rtol=1e-13, atol=0)
    T4.write_coef(y4, f4)
    z6 = T6.read_coef(f4)
    sd6 = T6.calc_sum_dof()
    low = sd6 <= 4
    assert np.allclose(z6[low], x6[low], rtol=1e-13, atol=0) and np.all(z6[~low] == 0)


def test_write_coef_formats_numbers_like_the_reference(tmp_path):
    """write_coef prints with an ostream at setprecision(14) in the default float
    format (src/Miscellaneous.cpp:108-127); the Python writer must give the same
    bytes for the same values, awkward ones included."""
    import os
    import subprocess
    vals = np.array([0.1, 1.0 / 3.0, -2.0 / 3.0, 1e-20, -1e-5, 123456789012345.0, 1.5e300, 5e-324, 0.0, -0.0,
                     100.0, 1e14, 1e15, 0.000123456789012345, 2.5, 3.5, 1.25e-7, -7.0])
    _, T = _space(4)
    x = np.zeros(T.n_dof_total)
    x[:len(vals)] = vals
    f = str(tmp_path / "c.txt")
    T.write_coef(x, f)
    src = tmp_path / "fmt.cpp"
    src.write_text("#include <iomanip>\n#include <iostream>\n#include <cstdio>\n"
                   "int main(){ double v; while (std::scanf(\"%la\", &v) == 1) "
                   "std::cout << std::setprecision(14) << v << '\\n'; return 0; }\n")
    exe = str(tmp_path / "fmt")
    subprocess.run(["g++", "-std=c++17", "-O0", str(src), "-o", exe], check=True, capture_output=True)
    hexes = "".join(float(v).hex() + "\n" for v in x)
    ref = subprocess.run([exe], input=hexes, capture_output=True, text=True, check=True).stdout
    with open(f) as fh:
        header = fh.readline()
        body = fh.read()
    assert header == f"4\t{T.n_dof_total}\n"
    assert body == ref
