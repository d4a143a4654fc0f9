"""AFEPack .mesh reader/writer: a written mesh reads back with the same topology,
marks and space (numbering, transforms)."""
import numpy as np

from tsemlib_gb300 import mesh, tsem


def test_write_read_round_trip(tmp_path):
    m = mesh.mark_box_boundary(mesh.kuhn_cube(2, 0.1, 3), [(0, 0.0), (0, 1.0)])
    f = str(tmp_path / "cube.mesh")
    mesh.write_afepack(m, f)
    r = mesh.read_afepack(f)
    for name in ("xyz", "tet_v", "tet_f", "face_v", "face_e", "edge_v", "mark_v", "mark_e", "mark_f", "femdof_v",
                 "femdof_e"):
        assert np.array_equal(getattr(r, name), getattr(m, name)), name
    a = tsem.TSEM(4, 6, m, lazy=True)
    b = tsem.TSEM(4, 6, r, lazy=True)
    for x, y in zip(a.transform(), b.transform()):
        assert np.array_equal(x, y)
