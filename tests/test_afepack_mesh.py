"""AFEPack .mesh reader/writer: a written mesh reads back with the same topology,
marks and space (numbering, transforms); the reference's own example meshes read
into a consistent topology, and the laplaceEig example runs on its mesh."""
import os

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


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_reference_example_meshes_read():
    """The reference's three example meshes read into a consistent topology: every
    tetrahedron's faces and edges are built from its own vertices, every mesh is a
    ball (V - E + F - T = 1), and the marks are the ones the examples impose on."""
    import os
    expect = {"ref_poisson_cube.mesh": (8, 6, [0, 1, 2]), "ref_laplace_cube.mesh": (8, 6, [0, 1]),
              "ref_helium_cube_atom.mesh": (None, 184, None)}
    for name, (nv, nt, marks) in expect.items():
        m = mesh.read_afepack(os.path.join(GOLDEN, name))
        assert m.nt == nt and (nv is None or m.nv == nv)
        assert m.nv - m.ne + m.nf - m.nt == 1
        for t in range(m.nt):
            vs = set(m.tet_v[t].tolist())
            for f in m.tet_f[t]:
                assert set(m.face_v[f].tolist()) <= vs
                for e in m.face_e[f]:
                    assert set(m.edge_v[e].tolist()) <= vs
        if marks is not None:
            assert sorted(np.unique(m.mark_f).tolist()) == marks
        # faces on the boundary of the domain are the faces of one tetrahedron only
        count = np.bincount(m.tet_f.ravel(), minlength=m.nf)
        assert np.all((count == 1) == (m.mark_f != 0))


def test_laplace_example_on_its_mesh_through_the_oracle():
    """examples/laplaceEig/laplaceEig.cpp on its own mesh (no refinement): zero
    boundary conditions on mark 1, inverse power from a random start, and the
    example's check against the first eigenvalue of the unit cube, 3 pi^2
    (laplaceEig.cpp:72-96), run through the AFEPack reader and the oracle.  The
    Rayleigh quotient stays above 3 pi^2 and its error falls spectrally with the
    order (1.1, 0.19, 1.0e-2, 2.5e-3, 3.7e-5 for p = 4..8)."""
    import oracle
    m = mesh.read_afepack(os.path.join(GOLDEN, "ref_laplace_cube.mesh"))
    errs = []
    for p in (4, 5, 6, 7, 8):
        S = oracle.Space(m, p, quad_q=p + 3)
        A, B = S.assemble("stiff"), S.assemble("mass")
        S.zero_bc(A, None, 1)
        S.zero_bc(B, None, 1)
        x = np.random.default_rng(1).uniform(0.0, 1.0, S.n_dof)
        S.zero_bc(None, x, 1)
        lam, x, it = oracle.inverse_power(A, B, x, 1e-12, 1000)
        assert it < 1000
        errs.append(lam - 3 * np.pi ** 2)
    assert all(e > 0 for e in errs)
    assert errs[-1] < 1e-4 and errs[-1] < 1e-4 * errs[0]
    assert all(b < a for a, b in zip(errs, errs[1:]))
