"""Copy TSEMLib's default quadrature tables into this folder as test fixtures.

TSEM<double>::init reads three tables by default (include/TetrahedralSEM.h:144-147,
src/QuadInfo.cpp:13-60): a 20-point 1-D rule, a 130-point 2-D rule (degree 26) and
a 923-point 3-D rule (degree 26), from include/quad_info/.  The tests read them
through tsem.read_quad_tables.

It also gathers the 1-D Gauss-Legendre tables that build_quad_info reads for a
collapsed rule of q points per direction (include/quad_info/qinfo_1d/qinfo_1d_order<q>,
src/QuadInfo.cpp:63-119; q = 2..64, one `abscissa weight` pair per line) into
qinfo_1d_orders.txt: a line `order q`, then that file's q lines.

Run in a checkout that has the reference available:

    python tests/golden/make_quad_tables.py /path/to/TSEMLib
"""
import os
import shutil
import sys

FILES = ["quad_info_1d_p38.dat", "quad_2d_deg26_n130.dat", "quad_3d_deg26_n923.dat"]


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_quad_tables.py <path of the TSEMLib checkout>")
    here = os.path.dirname(os.path.abspath(__file__))
    for f in FILES:
        shutil.copyfile(os.path.join(sys.argv[1], "include", "quad_info", f), os.path.join(here, f))
        print("wrote", os.path.join(here, f))
    out = []
    for q in range(2, 65):
        src = os.path.join(sys.argv[1], "include", "quad_info", "qinfo_1d", f"qinfo_1d_order{q}")
        lines = [ln for ln in open(src).read().splitlines() if ln.strip()]
        assert len(lines) == q, (q, len(lines))
        out.append(f"order {q}")
        out.extend(lines)
    with open(os.path.join(here, "qinfo_1d_orders.txt"), "w") as f:
        f.write("\n".join(out) + "\n")
    print("wrote", os.path.join(here, "qinfo_1d_orders.txt"))


if __name__ == "__main__":
    main()
