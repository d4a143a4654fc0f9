"""Pins of the CPU oracle (no GPU).

The reference ships no golden outputs for this path, so the oracle is pinned by
what the reference does hold: its face re-orientation table (tests/golden,
extracted from include/quad_info/Info_Interpolate_More), the global<->local
self-test it prints (src/BuildSpace.cpp:1228-1289), the quadrature weight sums it
prints (src/QuadInfo.cpp:85-118), the analytic eigenvalue check of
examples/laplaceEig/laplaceEig.cpp:96 and manufactured solutions.  The analytic
reference matrices are cross-checked against exact quadrature of the basis, and
the Rayleigh-Ritz step against LAPACK's dsygvx, the routine the reference calls
there (scipy's bundled LAPACK).
"""
import os

import numpy as np
import pytest

import oracle
from tsemlib_gb300 import mesh
from tsemlib_gb300 import manufactured as mf


def _cfg1_mesh(n, seed=1, jitter=0.1):
    m = mesh.kuhn_cube(n, jitter, seed)
    return mesh.mark_box_boundary(m, [(0, 0.0), (0, 1.0)])


@pytest.mark.parametrize("p", [4, 5, 6, 7, 8, 10])
def test_reference_matrices_match_quadrature(p):
    S = oracle.Space(_cfg1_mesh(1), p, quad_q=p + 3)
    q = S.quadrature()
    assert abs(q["w3"].sum() - 1) < 1e-13 and abs(q["w2"].sum() - 1) < 1e-13
    phi = np.array([S.basis_values(x) for x in q["x3"]])
    grad = np.array([S.basis_gradients(x) for x in q["x3"]])
    M_ref, pat = S.refmat(0)
    M_q = (phi.T * q["w3"]) @ phi / 6
    assert np.abs(M_ref - M_q).max() < 1e-14
    assert np.abs(M_q[~pat]).max() < 1e-14          # structural pattern covers all nonzeros
    dirs = [(1, 0, 0), (-1, 1, 0), (1, 0, -1), (0, 1, 0), (0, -1, 1), (0, 0, 1)]
    for k, d in enumerate(dirs):
        S_ref, pk = S.refmat(k + 1)
        D = grad @ np.array(d, float)
        S_q = (D.T * q["w3"]) @ D / 6
        assert np.abs(S_ref - S_q).max() < 1e-13 * max(1.0, np.abs(S_q).max())
        assert np.abs(S_q[~pk]).max() < 1e-13


def test_vertex_modes_are_barycentric():
    S = oracle.Space(_cfg1_mesh(1), 4, quad_q=3)
    for pt in [(0.1, 0.2, 0.3), (0.25, 0.25, 0.25), (0.6, 0.1, 0.05)]:
        v = S.basis_values(np.array(pt))
        assert np.allclose(v[:4], [1 - sum(pt), pt[0], pt[1], pt[2]], atol=1e-14)


def test_sizes_match_kuhn_formula():
    for n, p in [(2, 4), (3, 5)]:
        S = oracle.Space(_cfg1_mesh(n), p, quad_q=3)
        assert S.n_dof == mesh.dof_count(n, p)
        assert S.n_loc == (p + 1) * (p + 2) * (p + 3) // 6


def _face_mismatch(p, face_table=oracle.FACE_TABLE):
    """Largest difference, over the interior faces of a shuffled mesh and three points
    on each, between a random global function seen from the face's two tetrahedra."""
    m = mesh.shuffle_local_order(mesh.kuhn_cube(2, 0.15, 3), 7)
    S = oracle.Space(m, p, quad_q=3, face_table=face_table)
    g = S.geometry()
    assert np.all(np.bincount(g["type_face"], minlength=6) > 0)
    tn, ti, tv = S.transform()
    u = np.random.default_rng(0).standard_normal(S.n_dof)
    mask = np.arange(S.max_dep)[None, None, :] < tn[..., None]
    loc = (u[ti] * tv * mask).sum(-1)
    owners = {}
    for t in range(m.nt):
        for k in range(4):
            owners.setdefault(int(m.tet_f[t, k]), []).append(t)
    worst = 0.0
    for f, ts in owners.items():
        if len(ts) != 2:
            continue
        fv = m.xyz[m.face_v[f]]
        for bc in [(0.2, 0.3, 0.5), (0.6, 0.25, 0.15), (0.1, 0.7, 0.2)]:
            pt = bc[0] * fv[0] + bc[1] * fv[1] + bc[2] * fv[2]
            vals = []
            for t in ts:
                P = m.xyz[m.tet_v[t]]
                xh = np.linalg.solve((P[1:] - P[0]).T, pt - P[0])
                vals.append(S.basis_values(xh) @ loc[t])
            worst = max(worst, abs(vals[0] - vals[1]))
    return worst


@pytest.mark.parametrize("p", [4, 6, 8])
def test_global_functions_conform_across_faces(p):
    """All six face permutations and both edge orientations: the global function
    seen from the two tetrahedra of a face must agree on the face."""
    assert _face_mismatch(p) < 1e-12


def _write_face_table(path, t, M):
    """The library's derived table (tsem.face_table) in the layout of the
    reference's Info_Interpolate_More records."""
    nf = (M - 2) * (M - 3) // 2 + M - 2
    edge, face = {}, {}
    for v, d, k, e, i, x in zip(t["var"], t["dof"], t["kind"], t["edge_k"], t["index"], t["value"]):
        key = (int(v), int(d), int(e)) if k == 0 else (int(v), int(d))
        (edge if k == 0 else face).setdefault(key, []).append(f"{int(i)} {float(x):.17g}")
    out = [str(M)]
    for v in range(6):
        for d in range(nf):
            for e in range(3):
                ent = edge.get((v, d, e), [])
                out.append(" ".join([str(len(ent))] + ent))
        for d in range(nf):
            ent = face.get((v, d), [])
            out.append(" ".join([str(len(ent))] + ent))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


@pytest.mark.parametrize("p", [12, 13, 16])
def test_reference_face_table_loses_conformity_from_order_13(p, tmp_path):
    """The reference's Info_Interpolate_More leaves out coefficients from order 13 on
    (tests/golden/face_table_M16.txt is its M <= 16 prefix): with its table the
    global basis of order 13 jumps across faces by about 5e-6, of order 16 by about
    3e-5, where order 12 conforms to rounding.  The library derives its table from
    trace conformity, and with it every order conforms to rounding."""
    from tsemlib_gb300 import tsem
    ref = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "face_table_M16.txt")
    mine = str(tmp_path / "derived_M16.txt")
    _write_face_table(mine, tsem.face_table(16), 16)
    assert _face_mismatch(p, mine) < 1e-12
    w_ref = _face_mismatch(p, ref)
    if p <= 12:
        assert w_ref < 1e-12
    else:
        assert w_ref > 1e-7, w_ref


def test_transform_is_invertible_per_element():
    """Counterpart of the reference's random global->local->global self-test:
    restricted to an element's own DOFs the transform is a bijection."""
    m = mesh.shuffle_local_order(mesh.kuhn_cube(2, 0.1, 5), 11)
    S = oracle.Space(m, 6, quad_q=3)
    tn, ti, tv = S.transform()
    for e in range(0, m.nt, 5):
        dofs = np.unique(ti[e][np.arange(S.max_dep)[None, :] < tn[e][:, None]])
        assert dofs.size == S.n_loc
        T = np.zeros((S.n_loc, S.n_loc))
        pos = {d: i for i, d in enumerate(dofs)}
        for i in range(S.n_loc):
            for j in range(tn[e, i]):
                T[i, pos[ti[e, i, j]]] += tv[e, i, j]
        assert np.linalg.cond(T) < 1e8


@pytest.mark.parametrize("p", [4, 5])
def test_assembly_properties(p):
    m = _cfg1_mesh(2)
    S = oracle.Space(m, p, quad_q=4)
    A = S.assemble("stiff")
    Mm = S.assemble("mass")
    rp, c, v = A.arrays()
    assert all(c[rp[i]] == i for i in range(S.n_dof))        # diagonal first
    for i in range(S.n_dof):                                  # then strictly ascending
        assert np.all(np.diff(c[rp[i] + 1:rp[i + 1]]) > 0)
    dense = np.zeros((S.n_dof, S.n_dof))
    for i in range(S.n_dof):
        dense[i, c[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
    assert np.abs(dense - dense.T).max() < 1e-13 * np.abs(dense).max()
    lg, la = S.numbering()
    one = np.zeros(S.n_dof)
    one[la[lg[:m.nv]]] = 1.0                                  # vertex modes = barycentrics
    assert np.abs(A.matvec(one)).max() < 1e-12
    assert abs(one @ Mm.matvec(one) - 1.0) < 1e-12            # |unit cube|
    x = np.zeros(S.n_dof)
    x[la[lg[:m.nv]]] = m.xyz[:, 0]                            # u = x is exact
    assert abs(x @ A.matvec(x) - 1.0) < 1e-11


def test_poisson_manufactured_converges():
    errs = []
    for n, p in [(2, 4), (2, 5), (2, 6)]:
        S = oracle.Space(_cfg1_mesh(n), p, quad_q=p + 6)
        A = S.assemble("stiff")
        b = S.rhs(mf.f_cfg1)
        S.neumann(b, mf.neumann_cfg1, 2)
        S.dirichlet(A, b, mf.u_cfg1, True, 1)
        x, st = oracle.pcg(A, b, tol=1e-14, flag=1)
        assert st["status"] == 0
        errs.append(S.errors(x, mf.u_cfg1, mf.grad_cfg1))
    l2 = [e[0] for e in errs]
    h1 = [e[1] for e in errs]
    assert l2[0] > 4 * l2[1] > 16 * l2[2] and l2[2] < 1e-4
    assert h1[0] > 3 * h1[1] > 9 * h1[2]


def test_pmg_pcg_matches_jacobi_pcg():
    p = 4
    S = oracle.Space(_cfg1_mesh(2), p, quad_q=8)
    A = S.assemble("stiff")
    b = S.rhs(mf.f_cfg1)
    S.neumann(b, mf.neumann_cfg1, 2)
    S.dirichlet(A, b, mf.u_cfg1, True, 1)
    x1, s1 = oracle.pcg(A, b, tol=1e-14, flag=1)
    for step in (1, 2):
        P = oracle.PMG(A, p, S.sum_dof(), step)
        lv = P.levels()
        assert lv[-1] == (2 * 1 + 1) ** 3                     # p = 1 level: the vertices
        x2, s2 = oracle.pcg(A, b, tol=1e-14, flag=4, pmg=P, smooth=2)
        assert s2["iterations"] < s1["iterations"]
        assert np.abs(x1 - x2).max() < 1e-12


def test_laplace_eigenvalues_lobpcg_and_inverse_power():
    p = 4
    m = mesh.mark_all_boundary(mesh.kuhn_cube(2, 0.0, 0))
    S = oracle.Space(m, p, quad_q=4)
    A = S.assemble("stiff")
    B = S.assemble("mass")
    S.zero_bc(A, None, 1)
    S.zero_bc(B, None, 1)
    # boundary rows keep their diagonals: remove those decoupled modes by a shift
    rng = np.random.default_rng(1)
    X0 = rng.uniform(-1, 1, (4, S.n_dof))
    sd = S.sum_dof()
    bnd = np.zeros(S.n_dof, bool)
    lg, la = S.numbering()
    # eigenvalue of a decoupled boundary row is A_ii / B_ii; project the block off them
    X0[:, _boundary_dofs(S, m)] = 0.0
    lam, X, st = oracle.lobpcg(A, B, X0, tol=1e-9, max_it=300, precond=1)
    exact = np.pi ** 2 * np.array([3, 6, 6, 6])
    assert np.abs(lam - exact).max() / exact.max() < 1e-2   # N = 2, p = 4: discretisation error
    e, x, it = oracle.inverse_power(A, B, X0[0], tol=1e-10)
    assert abs(e - lam[0]) < 1e-7 * lam[0]


def _boundary_dofs(S, m):
    lg, la = S.numbering()
    out = []
    offs = [0, m.nv, m.nv + m.ne]
    marks = [m.mark_v, m.mark_e, m.mark_f]
    for d in range(3):
        for gidx in np.nonzero(marks[d])[0]:
            s = la[lg[offs[d] + gidx]]
            out.extend(range(s, s + S.n_dof_geo[d]))
    return np.array(out, dtype=np.int64)


@pytest.mark.parametrize("p", [4, 6, 8])
def test_interpolation_reproduces_polynomials_of_the_degree(p):
    """calc_interpolation (src/Interpolation.cpp:12-101) is exact for polynomials the
    space holds: vertex values, edge / face / interior projections together give back
    a degree-4 polynomial on a jittered mesh with shuffled local vertex orders."""
    def poly(q):
        x, y, z = q[..., 0], q[..., 1], q[..., 2]
        return x * x * y - 0.5 * z ** 4 + x * y * z + 0.3 * y * y * z * x - 2.0 * x + 1.0
    m = mesh.mark_all_boundary(mesh.shuffle_local_order(mesh.kuhn_cube(2, 0.1, 6), 7))
    S = oracle.Space(m, p, quad_q=p + 3)
    c = S.interpolation(poly)
    l2, _ = S.errors(c, poly, lambda q: np.zeros(q.shape))
    assert l2 <= 1e-13


def _pencil(m, seed, n=400):
    """Gram matrices of a random block S (n x m) against a 1-D Laplacian pencil
    (A tridiagonal stiffness, B tridiagonal mass): the shape of the projected
    problems LOBPCG forms."""
    rng = np.random.default_rng(seed)
    h = 1.0 / (n + 1)
    A = (np.diag(np.full(n, 2.0)) - np.diag(np.ones(n - 1), 1) - np.diag(np.ones(n - 1), -1)) / h
    B = (np.diag(np.full(n, 4.0)) + np.diag(np.ones(n - 1), 1) + np.diag(np.ones(n - 1), -1)) * h / 6
    S = rng.standard_normal((n, m))
    return S.T @ A @ S, S.T @ B @ S, S, A, B


@pytest.mark.parametrize("m,seed", [(3, 1), (3, 2), (12, 3), (48, 4)])
def test_rayleigh_ritz_matches_lapack_dsygvx(m, seed):
    """The reference solves its projected problem with LAPACKE_dsygvx(itype 1, 'V',
    'I', 'U', il = iu = 1) on 3 x 3 Grams (src/TSEMSolver.cpp:2179, 2349); the
    oracle's Rayleigh-Ritz (Jacobi on the B-scaled pencil) must give the same
    pairs.  LAPACK here is scipy's bundled build."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    ga, gb, *_ = _pencil(m, seed)
    theta, C = oracle.rayleigh_ritz(ga, gb)
    assert len(theta) == m
    # the reference's call: the smallest pair only
    w1, z1, found, _, info = lapack.dsygvx(ga, gb, itype=1, jobz="V", range="I", uplo="U", il=1, iu=1, abstol=-1.0)
    assert info == 0 and found == 1
    assert abs(theta[0] - w1[0]) <= 1e-12 * abs(w1[0])
    z = z1[:, 0]
    c = C[:, 0] * np.sign(C[:, 0] @ gb @ z)
    assert np.abs(c - z).max() <= 1e-9 * np.abs(z).max()
    # every pair
    w, Z, found, _, info = lapack.dsygvx(ga, gb, itype=1, jobz="V", range="I", uplo="U", il=1, iu=m, abstol=-1.0)
    assert info == 0 and found == m
    assert np.abs(theta - w[:m]).max() <= 1e-11 * np.abs(w[:m]).max()
    assert np.abs(C.T @ gb @ C - np.eye(m)).max() <= 1e-10
    gap = np.minimum(np.r_[np.inf, np.diff(w[:m])], np.r_[np.diff(w[:m]), np.inf]) / np.abs(w[:m]).max()
    for j in np.nonzero(gap > 1e-4)[0]:
        c = C[:, j] * np.sign(C[:, j] @ gb @ Z[:, j])
        assert np.abs(c - Z[:, j]).max() <= 1e-6 * np.abs(Z[:, j]).max(), j


def test_rayleigh_ritz_drops_a_dependent_direction_where_dsygvx_fails():
    """A basis column that lies in the span of the others makes GB singular:
    dsygvx reports it (info > n, the reference then stops its iteration), the
    oracle keeps the independent span and returns its Ritz pairs, which equal
    dsygvx's on that span."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    _, _, S, A, B = _pencil(6, 5)
    S = np.c_[S, S[:, 0] - 2.0 * S[:, 3]]
    ga, gb = S.T @ A @ S, S.T @ B @ S
    *_, info = lapack.dsygvx(ga, gb, itype=1, jobz="V", range="I", uplo="U", il=1, iu=7, abstol=-1.0)
    assert info > 7
    theta, C = oracle.rayleigh_ritz(ga, gb)
    assert len(theta) == 6
    w, *_ = lapack.dsygvx(ga[:6, :6], gb[:6, :6], itype=1, jobz="V", range="I", uplo="U", il=1, iu=6, abstol=-1.0)
    assert np.abs(theta - w[:6]).max() <= 1e-9 * np.abs(w[:6]).max()
