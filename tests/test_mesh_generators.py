"""The synthetic meshes the benchmark configurations are defined on (CPU only).

Kuhn cubes (configurations 1-3, serving): n^3 sub-cubes of 6 tetrahedra, interior
nodes moved by U(-0.1 h, 0.1 h) per coordinate, boundary nodes only along their
boundary planes, so the domain stays the unit cube; every tetrahedron keeps a
positive volume; (p n + 1)^3 DOFs.  The graded mesh of the Kohn-Sham configuration:
[-10, 10]^3 with 10 cells per half-axis whose widths grow by 1.15 away from the
origin, 20 per side, 1 030 301 DOFs at p = 5."""
import numpy as np
import pytest

from tsemlib_gb300 import mesh


def _volumes(m):
    P = m.xyz[m.tet_v]
    d = P[:, 1:] - P[:, :1]
    return np.einsum("ij,ij->i", d[:, 0], np.cross(d[:, 1], d[:, 2])) / 6.0


@pytest.mark.parametrize("n,seed", [(6, 1), (12, 2024)])
def test_jittered_kuhn_cube(n, seed):
    m0 = mesh.kuhn_cube(n)
    m = mesh.kuhn_cube(n, 0.1, seed)
    assert m.nt == 6 * n ** 3 and m.nv == (n + 1) ** 3
    assert np.array_equal(m.tet_v, m0.tet_v)
    h = 1.0 / n
    d = m.xyz - m0.xyz
    assert np.abs(d).max() <= 0.1 * h + 1e-15
    on_plane = (np.abs(m0.xyz) < 1e-12) | (np.abs(m0.xyz - 1.0) < 1e-12)
    assert np.all(d[on_plane] == 0.0)                  # the boundary planes stay put
    assert np.abs(d[~on_plane]).max() > 0.05 * h       # the rest does move
    assert np.all(m.xyz >= 0.0) and np.all(m.xyz <= 1.0)
    v0, v = _volumes(m0), _volumes(m)
    assert np.all(np.abs(v0) > 0) and np.all(np.sign(v) == np.sign(v0))
    assert abs(np.abs(v).sum() - 1.0) <= 1e-12
    # the boundary faces are exactly the faces on the cube's planes
    bf = m.boundary_faces()
    fv = m.xyz[m.face_v[bf]]
    assert np.all(np.any(np.all((np.abs(fv) < 1e-12) | (np.abs(fv - 1.0) < 1e-12), axis=1), axis=1))
    assert np.count_nonzero(bf) == 12 * n * n


@pytest.mark.parametrize("n,p,dofs", [(6, 4, 15625), (24, 6, 3048625), (16, 5, 531441)])
def test_configuration_dof_counts(n, p, dofs):
    assert mesh.dof_count(n, p) == dofs


def test_graded_kohn_sham_mesh():
    c = mesh.graded_coords(10, 1.15, 10.0)
    assert len(c) == 21 and abs(c[0] + 10.0) <= 1e-12 and abs(c[-1] - 10.0) <= 1e-12 and c[10] == 0.0
    assert np.allclose(c, -c[::-1], rtol=0, atol=1e-12)
    w = np.diff(c[10:])
    assert np.allclose(w[1:] / w[:-1], 1.15, rtol=1e-12)
    m = mesh.kuhn_cube(20, coords=c)
    assert m.nt == 6 * 20 ** 3 and mesh.dof_count(20, 5) == 1030301
    assert abs(np.abs(_volumes(m)).sum() - 20.0 ** 3) <= 1e-9


def _marks(m):
    return [m.mark_v.copy(), m.mark_e.copy(), m.mark_f.copy()]


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_flag_bm_cube_marks_the_cube_faces():
    """build_flag_bm(bnd_left, bnd_right) marks exactly the boundary of [L, R]^3:
    the jittered unit cube and the graded Kohn-Sham box."""
    m = mesh.kuhn_cube(4, 0.1, 3)
    a = _marks(mesh.flag_bm_cube(m, 0.0, 1.0))
    assert _same(a, _marks(mesh.mark_all_boundary(m)))
    c = mesh.graded_coords(5, 1.15, 10.0)
    m = mesh.kuhn_cube(10, coords=c)
    a = _marks(mesh.flag_bm_cube(m, -10.0, 10.0))
    assert _same(a, _marks(mesh.mark_all_boundary(m)))
    # a smaller cube inside marks only the geometries on its planes, boundary ones none
    m = mesh.kuhn_cube(4)
    mesh.flag_bm_cube(m, 0.25, 0.75)
    pts = m.xyz[m.mark_v == 1]
    assert len(pts) > 0 and np.all(np.any((np.abs(pts - 0.25) < 1e-12) | (np.abs(pts - 0.75) < 1e-12), axis=1))
    assert np.all(m.mark_f[m.boundary_faces()] == 0)


def test_flag_bm_cube_in_a_rotated_frame():
    """build_flag_bm(L, R, axis): the cube [-1, 1]^3 turned by R is marked on its own
    boundary when the axes are R's columns."""
    t = 0.3
    Rz = np.array([[np.cos(t), -np.sin(t), 0], [np.sin(t), np.cos(t), 0], [0, 0, 1]])
    Rx = np.array([[1, 0, 0], [0, np.cos(2 * t), -np.sin(2 * t)], [0, np.sin(2 * t), np.cos(2 * t)]])
    R = Rz @ Rx
    m = mesh.kuhn_cube(3, coords=np.linspace(-1.0, 1.0, 4))
    m.xyz = m.xyz @ R.T
    a = _marks(mesh.flag_bm_cube(m, -1.0, 1.0, axis=R.T))
    b = _marks(mesh.mark_all_boundary(m))
    assert _same(a, b) and np.count_nonzero(a[2]) == 6 * 2 * 3 * 3
    c = _marks(mesh.flag_bm_cube(m, -1.0, 1.0))          # without the axes the test misses
    assert not np.array_equal(c[2], b[2])


def test_flag_bm_ball_marks_the_sphere():
    """build_flag_bm(radius): vertices on the sphere, and edges and faces whose
    vertices all are.  A cube mesh mapped radially onto the unit ball has its
    boundary vertices on the sphere."""
    m = mesh.kuhn_cube(4, coords=np.linspace(-1.0, 1.0, 5))
    r_inf = np.abs(m.xyz).max(axis=1)
    scale = np.where(r_inf > 0, r_inf / np.maximum(np.linalg.norm(m.xyz, axis=1), 1e-300), 0.0)
    m.xyz = m.xyz * scale[:, None]
    mesh.flag_bm_ball(m, 1.0)
    bnd = m.boundary_faces()
    on_sphere = np.zeros(m.nv, bool)
    on_sphere[m.face_v[bnd].ravel()] = True
    assert np.array_equal(m.mark_v == 1, on_sphere)
    assert np.all(m.mark_f[bnd] == 1)
    assert np.array_equal(m.mark_f == 1, np.all(on_sphere[m.face_v], axis=1))
    assert np.array_equal(m.mark_e == 1, np.all(on_sphere[m.edge_v], axis=1))
