"""Tetrahedral meshes with AFEPack-style topology.

TSEMLib takes its mesh from AFEPack (``RegularMesh<3>``, used through
``mesh.geometry(dim, i).vertex(k)`` / ``.boundary(k)`` / ``.boundaryMark()`` and
``mesh.point(i)``; see src/BuildSpace.cpp:436-546 and src/Discretize.cpp:109-118)
and its DOF ordering from an AFEPack P2 ``FEMSpace`` (src/BuildSpace.cpp:906-913).
This module builds the same information as plain arrays:

* ``tet_v[t][k]``: vertex k of tetrahedron t; ``tet_f[t][k]``: the face opposite it;
* ``face_v[f][k]``: vertex k of face f; ``face_e[f][k]``: the edge opposite it;
* ``edge_v[e]``: the two vertices of edge e;
* boundary marks per vertex / edge / face (0 = interior);
* ``femdof_v`` / ``femdof_e``: the number the P2 space gives each vertex and
  edge.  AFEPack numbers DOFs as it first meets them while walking the elements;
  the default here walks the tetrahedra in order, visiting vertices 0..3 and then
  edges 01, 02, 03, 12, 13, 23 of each.  A caller holding the real AFEPack order
  passes it instead.

It also generates the synthetic meshes the benchmarks use: Kuhn-split cubes
(6 tetrahedra per sub-cube) with seeded node jitter, and the graded cube.
"""
from __future__ import annotations

import dataclasses
import itertools

import numpy as np

# local edge k of a tetrahedron joins vertices (EDGE_A[k], EDGE_B[k]): E01 E02 E03 E12 E13 E23
EDGE_A = np.array([0, 0, 0, 1, 1, 2])
EDGE_B = np.array([1, 2, 3, 2, 3, 3])
# local face k is opposite vertex k; its vertices in the reference's order
# (src/BuildSpace.cpp:505-508)
FACE_PTS = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])


@dataclasses.dataclass
class TetMesh:
    xyz: np.ndarray          # [nv, 3] float64
    tet_v: np.ndarray        # [nt, 4] int32
    tet_f: np.ndarray        # [nt, 4] int32
    face_v: np.ndarray       # [nf, 3] int32
    face_e: np.ndarray       # [nf, 3] int32
    edge_v: np.ndarray       # [ne, 2] int32
    femdof_v: np.ndarray     # [nv] int32
    femdof_e: np.ndarray     # [ne] int32
    mark_v: np.ndarray       # [nv] int32
    mark_e: np.ndarray       # [ne] int32
    mark_f: np.ndarray       # [nf] int32

    @property
    def nv(self):
        return int(self.xyz.shape[0])

    @property
    def ne(self):
        return int(self.edge_v.shape[0])

    @property
    def nf(self):
        return int(self.face_v.shape[0])

    @property
    def nt(self):
        return int(self.tet_v.shape[0])

    def boundary_faces(self):
        """Faces that belong to exactly one tetrahedron."""
        cnt = np.bincount(self.tet_f.ravel(), minlength=self.nf)
        return cnt == 1


def _first_occurrence_unique(keys: np.ndarray):
    """Unique rows numbered by first appearance.  Returns (first_index, inverse)."""
    uniq, first, inv = np.unique(keys, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    return first[order], rank[inv.ravel()]


def build_topology(xyz: np.ndarray, tet_v: np.ndarray) -> TetMesh:
    """Number edges and faces by first appearance and fill the AFEPack relations."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    tet_v = np.ascontiguousarray(tet_v, dtype=np.int64)
    nt = tet_v.shape[0]
    # edges
    ea, eb = tet_v[:, EDGE_A], tet_v[:, EDGE_B]            # [nt, 6]
    ekey = np.stack([np.minimum(ea, eb), np.maximum(ea, eb)], axis=-1).reshape(-1, 2)
    efirst, eid = _first_occurrence_unique(ekey)
    eid = eid.reshape(nt, 6)
    edge_v = np.stack([ea.ravel()[efirst], eb.ravel()[efirst]], axis=1)
    # faces
    fv = tet_v[:, FACE_PTS]                                 # [nt, 4, 3]
    fkey = np.sort(fv, axis=-1).reshape(-1, 3)
    ffirst, fid = _first_occurrence_unique(fkey)
    tet_f = fid.reshape(nt, 4)
    face_v = fv.reshape(-1, 3)[ffirst]
    # edge opposite face vertex k joins the other two
    nf = face_v.shape[0]
    nv = xyz.shape[0]
    code = np.minimum(edge_v[:, 0], edge_v[:, 1]) * nv + np.maximum(edge_v[:, 0], edge_v[:, 1])
    sorter = np.argsort(code)
    face_e = np.empty((nf, 3), dtype=np.int64)
    for k in range(3):
        a = face_v[:, (k + 1) % 3]
        b = face_v[:, (k + 2) % 3]
        c = np.minimum(a, b) * nv + np.maximum(a, b)
        pos = np.searchsorted(code, c, sorter=sorter)
        face_e[:, k] = sorter[pos]
    # canonical P2 DOF order: walk tets, vertices then edges, number at first sight
    walk = np.concatenate([tet_v, eid + nv], axis=1).reshape(-1)
    _, first = np.unique(walk, return_index=True)
    keys_sorted = walk[np.sort(first)]
    femdof = np.empty(nv + edge_v.shape[0], dtype=np.int64)
    femdof[keys_sorted] = np.arange(keys_sorted.size)
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    z = lambda n: np.zeros(n, dtype=np.int32)
    return TetMesh(xyz=xyz, tet_v=i32(tet_v), tet_f=i32(tet_f), face_v=i32(face_v), face_e=i32(face_e),
                   edge_v=i32(edge_v), femdof_v=i32(femdof[:nv]), femdof_e=i32(femdof[nv:]),
                   mark_v=z(nv), mark_e=z(edge_v.shape[0]), mark_f=z(nf))


def kuhn_cube(n: int, jitter: float = 0.0, seed: int = 0, coords=None) -> TetMesh:
    """Unit cube split into n^3 sub-cubes of 6 Kuhn tetrahedra each.

    ``coords`` optionally gives the n+1 grid coordinates per axis (graded meshes).
    Interior nodes move by U(-jitter*h, jitter*h) per coordinate; boundary nodes
    move only along the boundary so the domain stays a box.
    """
    if coords is None:
        coords = np.linspace(0.0, 1.0, n + 1)
    coords = np.asarray(coords, dtype=np.float64)
    g = np.stack(np.meshgrid(coords, coords, coords, indexing="ij"), axis=-1).reshape(-1, 3)
    idx = lambda i, j, k: (i * (n + 1) + j) * (n + 1) + k
    I, J, K = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    tets = []
    for perm in itertools.permutations(range(3)):
        off = np.zeros(3, dtype=np.int64)
        verts = [idx(I, J, K)]
        for ax in perm:
            off[ax] += 1
            verts.append(idx(I + off[0], J + off[1], K + off[2]))
        tets.append(np.stack(verts, axis=1))
    # cube-major order: the 6 tetrahedra of a sub-cube are consecutive
    tet_v = np.stack(tets, axis=1).reshape(-1, 4)
    xyz = g.copy()
    if jitter > 0:
        rng = np.random.default_rng(seed)
        h = np.diff(coords)
        # local spacing per node and axis: the smaller adjacent cell width
        hl = np.minimum(np.concatenate([[h[0]], h]), np.concatenate([h, [h[-1]]]))
        ii = np.arange(n + 1)
        hn = np.stack(np.meshgrid(hl, hl, hl, indexing="ij"), axis=-1).reshape(-1, 3)
        on_bnd = np.stack(np.meshgrid(ii, ii, ii, indexing="ij"), axis=-1).reshape(-1, 3)
        on_bnd = (on_bnd == 0) | (on_bnd == n)
        d = rng.uniform(-jitter, jitter, size=xyz.shape) * hn
        d[on_bnd] = 0.0
        xyz = xyz + d
    return build_topology(xyz, tet_v)


def graded_coords(n_half: int, ratio: float, half_width: float) -> np.ndarray:
    """Symmetric grid coordinates on [-half_width, half_width]: n_half cells per
    half-axis with widths growing geometrically by ``ratio`` away from 0."""
    w = ratio ** np.arange(n_half)
    w = w / w.sum() * half_width
    pos = np.concatenate([[0.0], np.cumsum(w)])
    return np.concatenate([-pos[::-1], pos[1:]])


def mark_box_boundary(m: TetMesh, dirichlet_planes, other_mark: int = 2, tol: float = 1e-12,
                      lo=0.0, hi=1.0) -> TetMesh:
    """Boundary marks for a box: geometries lying on one of ``dirichlet_planes``
    ((axis, value) pairs) get mark 1, the rest of the boundary ``other_mark``."""
    bface = m.boundary_faces()
    bvert = np.zeros(m.nv, dtype=bool)
    bvert[m.face_v[bface].ravel()] = True
    bedge = np.zeros(m.ne, dtype=bool)
    bedge[m.face_e[bface].ravel()] = True

    def on_planes(vertex_sets):
        res = np.zeros(vertex_sets.shape[0], dtype=bool)
        for ax, val in dirichlet_planes:
            c = m.xyz[vertex_sets, ax]
            res |= np.all(np.abs(c - val) < tol, axis=1)
        return res

    mv = np.where(bvert, other_mark, 0)
    me = np.where(bedge, other_mark, 0)
    mf = np.where(bface, other_mark, 0)
    if dirichlet_planes:
        mv[bvert & on_planes(np.arange(m.nv)[:, None])] = 1
        me[bedge & on_planes(m.edge_v)] = 1
        mf[bface & on_planes(m.face_v)] = 1
    m.mark_v = mv.astype(np.int32)
    m.mark_e = me.astype(np.int32)
    m.mark_f = mf.astype(np.int32)
    return m


def mark_all_boundary(m: TetMesh, mark: int = 1) -> TetMesh:
    bface = m.boundary_faces()
    m.mark_f = np.where(bface, mark, 0).astype(np.int32)
    mv = np.zeros(m.nv, dtype=np.int32)
    mv[m.face_v[bface].ravel()] = mark
    me = np.zeros(m.ne, dtype=np.int32)
    me[m.face_e[bface].ravel()] = mark
    m.mark_v, m.mark_e = mv, me
    return m


def _barycenters(m: TetMesh):
    """Barycenters of the vertices, edges and faces (the point each geometry is
    tested at by TSEMLib's build_flag_bm, point_ref_mesh, src/BuildSpace.cpp:439-465)."""
    return m.xyz, m.xyz[m.edge_v].mean(axis=1), m.xyz[m.face_v].mean(axis=1)


def _set_marks(m: TetMesh, fv, fe, ff, mark: int) -> TetMesh:
    m.mark_v = np.where(fv, mark, 0).astype(np.int32)
    m.mark_e = np.where(fe, mark, 0).astype(np.int32)
    m.mark_f = np.where(ff, mark, 0).astype(np.int32)
    return m


def flag_bm_cube(m: TetMesh, bnd_left: float, bnd_right: float, axis=None, mark: int = 1,
                 tol: float = 1e-12) -> TetMesh:
    """build_flag_bm(bnd_left, bnd_right[, axis]) (src/Discretize.cpp:26-44, 79-104):
    a vertex, edge or face gets `mark` when its barycenter lies on a face of the cube
    [bnd_left, bnd_right]^3 (some coordinate within tol of bnd_left or bnd_right;
    is_on_boundary, :2066-2077), every other geometry 0.  With ``axis`` (three row
    vectors, axis[i] = the i-th axis of a rotated frame) the coordinates are the
    barycenter's inner products with those axes.  The library reads the marks
    from the mesh, so this is applied before the space is built."""
    A = np.eye(3) if axis is None else np.asarray(axis, dtype=np.float64).reshape(3, 3)

    def on(pts):
        c = pts @ A.T
        return np.any((np.abs(c - bnd_left) < tol) | (np.abs(c - bnd_right) < tol), axis=1)

    pv, pe, pf = _barycenters(m)
    return _set_marks(m, on(pv), on(pe), on(pf), mark)


def flag_bm_ball(m: TetMesh, radius: float, mark: int = 1, tol: float = 1e-12) -> TetMesh:
    """build_flag_bm(radius) (src/Discretize.cpp:47-77): a vertex gets `mark` when
    its distance from the origin is within tol of radius (:2080-2085), an edge or a
    face when all its vertices have it (faces and edges whose vertices all lie on the
    sphere, inside the ball as well), every other geometry 0."""
    fv = np.abs(np.linalg.norm(m.xyz, axis=1) - radius) < tol
    return _set_marks(m, fv, np.all(fv[m.edge_v], axis=1), np.all(fv[m.face_v], axis=1), mark)


def dof_count(n: int, p: int) -> int:
    """Number of DOFs of order p on an n^3 Kuhn cube: (p n + 1)^3."""
    return (p * n + 1) ** 3


def shuffle_local_order(m: TetMesh, seed: int = 0) -> TetMesh:
    """Same geometry with every tetrahedron's vertex list randomly permuted.

    Kuhn meshes orient every shared face identically; shuffled local orders make
    all six face permutations and both edge orientations appear."""
    rng = np.random.default_rng(seed)
    perm = np.argsort(rng.random((m.nt, 4)), axis=1)
    tv = np.take_along_axis(m.tet_v.astype(np.int64), perm, axis=1)
    out = build_topology(m.xyz, tv)
    return out


def write_afepack(m: TetMesh, filename: str) -> None:
    """Write a mesh in AFEPack's .mesh layout: the points, then for dimensions 0..3
    the geometries, each as its index, its vertex list and its boundary list (both
    prefixed by their length) and its boundary mark."""
    with open(filename, "w") as f:
        f.write(f"{m.nv}\n")
        for p in m.xyz:
            f.write(f"{p[0]:.17g}\t{p[1]:.17g}\t{p[2]:.17g}\n")
        f.write("\n\n")
        f.write(f"{m.nv}\n")
        for i in range(m.nv):
            f.write(f"{i}\n1\t{i}\n1\t{i}\n{int(m.mark_v[i])}\n")
        f.write("\n\n")
        f.write(f"{m.ne}\n")
        for i in range(m.ne):
            a, b = m.edge_v[i]
            f.write(f"{i}\n2\t{a}\t{b}\n2\t{a}\t{b}\n{int(m.mark_e[i])}\n")
        f.write("\n\n")
        f.write(f"{m.nf}\n")
        for i in range(m.nf):
            v, e = m.face_v[i], m.face_e[i]
            f.write(f"{i}\n3\t{v[0]}\t{v[1]}\t{v[2]}\n3\t{e[0]}\t{e[1]}\t{e[2]}\n{int(m.mark_f[i])}\n")
        f.write("\n\n")
        f.write(f"{m.nt}\n")
        for i in range(m.nt):
            v, fc = m.tet_v[i], m.tet_f[i]
            f.write(f"{i}\n4\t{v[0]}\t{v[1]}\t{v[2]}\t{v[3]}\n4\t{fc[0]}\t{fc[1]}\t{fc[2]}\t{fc[3]}\n0\n")


def read_afepack(filename: str) -> TetMesh:
    """Read AFEPack's .mesh layout (the format of TSEMLib's example meshes): points,
    then per dimension 0..3 the geometries with their vertex lists, boundary lists
    (edges of a face opposite its vertices, faces of a tetrahedron opposite its
    vertices) and boundary marks.  The P2 DOF order is the default walk of
    build_topology (AFEPack's own order needs AFEPack; pass it in femdof_v/_e)."""
    with open(filename) as f:
        tok = f.read().split()
    pos = 0

    def nxt():
        nonlocal pos
        pos += 1
        return tok[pos - 1]

    nv = int(nxt())
    xyz = np.array([[float(nxt()) for _ in range(3)] for _ in range(nv)])
    geo = []
    for dim in range(4):
        n = int(nxt())
        verts, bnds, marks = [], [], []
        for _ in range(n):
            nxt()                                   # index
            k = int(nxt())
            verts.append([int(nxt()) for _ in range(k)])
            k = int(nxt())
            bnds.append([int(nxt()) for _ in range(k)])
            marks.append(int(nxt()))
        geo.append((verts, bnds, marks))
    tet_v = np.array(geo[3][0], dtype=np.int64)
    m = build_topology(xyz, tet_v)
    # keep the file's own numbering of edges and faces and its relations
    m.edge_v = np.ascontiguousarray(geo[1][0], dtype=np.int32)
    m.face_v = np.ascontiguousarray(geo[2][0], dtype=np.int32)
    m.face_e = np.ascontiguousarray(geo[2][1], dtype=np.int32)
    m.tet_f = np.ascontiguousarray(geo[3][1], dtype=np.int32)
    m.mark_v = np.ascontiguousarray(geo[0][2], dtype=np.int32)
    m.mark_e = np.ascontiguousarray(geo[1][2], dtype=np.int32)
    m.mark_f = np.ascontiguousarray(geo[2][2], dtype=np.int32)
    # P2 DOF order walk over the file's numbering: tets in order, vertices then edges
    ekey = {}
    for i, (a, b) in enumerate(m.edge_v):
        ekey[(min(a, b), max(a, b))] = i
    order = {}
    for t in range(m.nt):
        v = m.tet_v[t]
        for k in range(4):
            order.setdefault(("v", int(v[k])), len(order))
        for k in range(6):
            a, b = int(v[EDGE_A[k]]), int(v[EDGE_B[k]])
            order.setdefault(("e", ekey[(min(a, b), max(a, b))]), len(order))
    m.femdof_v = np.array([order[("v", i)] for i in range(m.nv)], dtype=np.int32)
    m.femdof_e = np.array([order[("e", i)] for i in range(m.ne)], dtype=np.int32)
    return m
