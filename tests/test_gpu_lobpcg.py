"""Block LOBPCG on the GPU (TSEMSolver::solve_LOBPCG, src/TSEMSolver.cpp:2225-2406)
against a dense FP64 generalized eigensolve, the oracle's LOBPCG and the analytic
Dirichlet spectrum pi^2 (i^2 + j^2 + k^2) of the unit cube."""
import numpy as np
import pytest

import oracle
from tsemlib_gb300 import mesh, tsem

pytestmark = pytest.mark.gpu

# pi^2 (i^2 + j^2 + k^2), i, j, k >= 1, ascending with multiplicity
ANALYTIC = np.sort([np.pi ** 2 * (i * i + j * j + k * k)
                    for i in range(1, 6) for j in range(1, 6) for k in range(1, 6)])


def _eig_problem(n, p, jitter=0.0):
    m = mesh.mark_all_boundary(mesh.kuhn_cube(n, jitter, 1))
    T = tsem.TSEM(p, p + 2, m)
    A = T.stiff_matrix.copy()
    M = T.mass_matrix.copy()
    T.impose_zero_boundary_condition(A, None, 1)
    T.impose_zero_boundary_condition(M, None, 1)
    return T, A, M


def _initial_block(T, k, seed=7):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1.0, 1.0, (T.n_dof_total, k))
    for j in range(k):
        col = np.ascontiguousarray(X[:, j])
        T.impose_zero_boundary_condition(None, col, 1)
        X[:, j] = col
    return X


def _interior_dense(T, A, M):
    """Dense FP64 pencil on the DOFs that are not Dirichlet DOFs."""
    import scipy.linalg as sla
    import scipy.sparse as sps
    n = T.n_dof_total
    probe = np.ones(n)
    T.impose_zero_boundary_condition(None, probe, 1)
    keep = np.nonzero(probe)[0]
    rp, c, v = A.arrays()
    Ad = sps.csr_matrix((v, c, rp), shape=(n, n))[keep][:, keep].toarray()
    rp, c, v = M.arrays()
    Md = sps.csr_matrix((v, c, rp), shape=(n, n))[keep][:, keep].toarray()
    return sla.eigh(Ad, Md, eigvals_only=True)


@pytest.mark.parametrize("jitter", [0.0, 0.1])
def test_lobpcg_plain_matches_dense_and_oracle(jitter):
    T, A, M = _eig_problem(2, 4, jitter)
    k, want = 8, 6
    X = _initial_block(T, k)
    sol = tsem.TSEMSolver()
    sol.init_PMG(A, 4, T.calc_sum_dof(), order_step=2, smoother="gs")
    # residual 1e-8 (the block products run on the FP32 pipe with (hi, lo) operands; the
    # eigenvalue error is of the order of the squared residual)
    lam, st = sol.solve_LOBPCG(T, X, A, M, tol=1e-8, max_step=300, n_want=want)
    assert st["status"] == "OK", st
    ref = _interior_dense(T, A, M)[:want]
    assert np.allclose(lam[:want], ref, rtol=1e-9, atol=0), (lam[:want], ref)
    # M-orthonormal Ritz vectors
    rp, c, v = M.arrays()
    Mo = oracle.Csr.from_arrays(rp, c, v)
    MX = np.stack([Mo.matvec(X[:, j]) for j in range(k)], axis=1)
    assert np.abs(X.T @ MX - np.eye(k)).max() < 1e-9
    # the oracle's block LOBPCG from the same start
    rp, c, v = A.arrays()
    Ao = oracle.Csr.from_arrays(rp, c, v)
    lo, _, so = oracle.lobpcg(Ao, Mo, _initial_block(T, k).T, tol=1e-9, max_it=300, precond=1)
    assert np.allclose(lam[:want], lo[:want], rtol=1e-9, atol=0), (lam[:want], lo[:want])


def test_lobpcg_mixed_preconditioner_reaches_analytic_spectrum():
    """Mixed solver: FP32 matrix-free V-cycle preconditioner, FP64 Gram and Ritz.
    N = 4, p = 6 resolves the lowest ten modes of pi^2 (i^2 + j^2 + k^2) to < 1e-7
    (discretisation error; the oracle's eigenvalues of the same pencil differ from
    the analytic ones by 2e-10 .. 7.5e-8)."""
    T, A, M = _eig_problem(4, 6)
    k, want = 12, 10
    X = _initial_block(T, k)
    mx = tsem.MixedSolver(T, A, 1, order_step=2)
    lam, st = mx.solve_LOBPCG(X, M, tol=1e-8, max_step=300, n_want=want)
    assert st["status"] == "OK", st
    # the Jacobi of every Rayleigh-Ritz step ends by its own test, well before the cap
    assert 1 <= st["jacobi_sweeps"] < 30, st
    rel = np.abs(lam[:want] - ANALYTIC[:want]) / ANALYTIC[:want]
    assert rel.max() < 1e-7, rel
    # same pencil, plain FP64 preconditioner: the eigenvalues agree to the solve tolerance
    sol = tsem.TSEMSolver()
    sol.init_PMG(A, 6, T.calc_sum_dof(), order_step=2, smoother="chebyshev")
    lam64, st64 = sol.solve_LOBPCG(T, _initial_block(T, k), A, M, tol=1e-8, max_step=300, n_want=want)
    assert st64["status"] == "OK", st64
    assert np.allclose(lam[:want], lam64[:want], rtol=1e-11, atol=0)


def test_lobpcg_single_vector_and_list_input():
    """k = 1 (the reference's single-vector form) with the block given as a list."""
    T, A, M = _eig_problem(2, 4)
    x = [_initial_block(T, 1)[:, 0].copy()]
    sol = tsem.TSEMSolver()
    sol.init_PMG(A, 4, T.calc_sum_dof(), order_step=2, smoother="gs")
    lam, st = sol.solve_LOBPCG(T, x, A, M, tol=1e-8, max_step=300)
    assert st["status"] == "OK", st
    ref = _interior_dense(T, A, M)[0]
    assert abs(lam[0] - ref) <= 1e-10 * ref
    assert abs(lam[0] - 3 * np.pi ** 2) / (3 * np.pi ** 2) < 1e-2


def test_lobpcg_many_pairs_on_a_small_mesh_both_forms():
    """A block of 28 for 24 pairs on a p = 2 mesh of 4913 interior DOFs: the block
    spans a large part of the low spectrum, where the preconditioned residuals lie
    nearly inside span(X).  Both forms must converge (the residuals are projected
    against X before the Rayleigh-Ritz step, and the plain V-cycle starts from zero
    for every column) and agree on the eigenvalues."""
    T, A, M = _eig_problem(9, 2, jitter=0.1)
    k, want = 28, 24
    sol = tsem.TSEMSolver()
    sol.init_PMG(A, 2, T.calc_sum_dof(), order_step=2, smoother="chebyshev")
    lam_p, st_p = sol.solve_LOBPCG(T, _initial_block(T, k), A, M, tol=1e-8, max_step=300, n_want=want,
                                   smooth_step=4)
    mx = tsem.MixedSolver(T, A, 1, order_step=2)
    lam_m, st_m = mx.solve_LOBPCG(_initial_block(T, k), M, tol=1e-8, max_step=300, n_want=want)
    assert st_p["status"] == "OK" and st_p["iterations"] < 150, st_p
    assert st_m["status"] == "OK" and st_m["iterations"] < 150, st_m
    assert np.abs(lam_p[:want] - lam_m[:want]).max() <= 1e-7 * np.abs(lam_p[:want]).max()
    assert np.all(np.diff(lam_m[:want]) >= -1e-9 * lam_m[want - 1])


def test_lobpcg_pencil_with_unrelated_patterns():
    """A and M whose patterns hold neither the other (the mass pattern holds the
    stiffness one; here one small symmetric pair of the stiffness pattern is taken out
    of M), so the block products run as two passes instead of one: the eigenvalues
    still match the dense FP64 solve of the same pencil."""
    T, A, M = _eig_problem(2, 4)
    rp, c, v = M.arrays()
    ra, ca, _ = A.arrays()
    n = len(rp) - 1
    in_a = set()
    for i in range(n):
        for j in ca[ra[i]:ra[i + 1]]:
            in_a.add((i, int(j)))
    # the smallest off-diagonal M entry of an interior row whose column is in A's pattern
    probe = np.ones(n)
    T.impose_zero_boundary_condition(None, probe, 1)
    best = None
    for i in np.nonzero(probe)[0]:
        for t in range(rp[i] + 1, rp[i + 1]):
            j = int(c[t])
            if j != i and probe[j] != 0 and (i, j) in in_a and v[t] != 0.0:
                if best is None or abs(v[t]) < best[2]:
                    best = (int(i), j, abs(v[t]))
    assert best is not None
    i0, j0, _ = best
    keep = np.ones(len(c), bool)
    for r, col in ((i0, j0), (j0, i0)):
        t = rp[r] + int(np.nonzero(c[rp[r]:rp[r + 1]] == col)[0][0])
        keep[t] = False
    counts = np.array([keep[rp[i]:rp[i + 1]].sum() for i in range(n)])
    rp2 = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    B = tsem.SparseMatrix.from_arrays(rp2, c[keep].astype(np.int32), v[keep])
    k, want = 8, 6
    sol = tsem.TSEMSolver()
    sol.init_PMG(A, 4, T.calc_sum_dof(), order_step=2, smoother="gs")
    X = _initial_block(T, k)
    lam, st = sol.solve_LOBPCG(T, X, A, B, tol=1e-8, max_step=300, n_want=want)
    assert st["status"] == "OK", st
    ref = _interior_dense(T, A, B)[:want]
    assert np.allclose(lam[:want], ref, rtol=1e-9, atol=0), (lam[:want], ref)
