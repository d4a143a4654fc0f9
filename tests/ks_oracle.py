"""TEST INFRASTRUCTURE ONLY: the helium Kohn-Sham loop of tsemlib_gb300.ks restated
on the CPU oracle (FP64 throughout), for a reference energy on a small mesh.

Same physics and the same fixed point as ks.helium: V = V_ext + V_H + V_x with the
smoothed -Z/r, LDA exchange, the Hamiltonian 1/2 K + M_V (build_mass_V_matrix,
src/Discretize.cpp:668-843), block LOBPCG for the lowest states (p-multigrid
preconditioner of K), the density sum_j occ_j psi_j^2 (calc_density,
src/PointInfo.cpp:72-91) mixed linearly, the Hartree potential from the Poisson
problem with the multipole boundary data of SCFIteration.cpp:70-153 imposed as
SCFIteration.cpp:170-176 does (a fresh copy of the stiffness matrix, the matrix
modified), and the energy n_occ eps_0 - E_H + int (eps_x - V_x) rho of the input
density.  The two loops take different paths (preconditioners, eigen tolerances per
step) to the same self-consistent density, so their converged energies agree to the
SCF tolerance.
"""
import numpy as np
import scipy.sparse as sp

import oracle
from tsemlib_gb300 import ks


def _to_scipy(A):
    rp, c, v = A.arrays()
    return sp.csr_matrix((v, c, rp), shape=(len(rp) - 1, len(rp) - 1))


def _from_scipy(B):
    """deal.II row convention for the oracle: diagonal first, then ascending columns"""
    B = B.tocsr()
    B.sort_indices()
    rp, c, v = B.indptr.astype(np.int64), B.indices.astype(np.int32), B.data.copy()
    for i in range(B.shape[0]):
        s, e = rp[i], rp[i + 1]
        cols, vals = c[s:e].copy(), v[s:e].copy()
        d = np.nonzero(cols == i)[0]
        order = np.concatenate([d, np.setdiff1d(np.arange(e - s), d)])
        c[s:e], v[s:e] = cols[order], vals[order]
    return oracle.Csr.from_arrays(rp, c, v)


class _Eval:
    """FE function values at the element quadrature points through T_e"""

    def __init__(self, S):
        q = S.quadrature()
        self.phi = np.stack([S.basis_values(x) for x in q["x3"]])          # [nq, n_loc]
        self.tn, self.ti, self.tv = S.transform()

    def __call__(self, x):
        ti = np.where(self.ti >= 0, self.ti, 0)
        loc = (x[ti] * self.tv * (np.arange(self.ti.shape[2])[None, None, :] < self.tn[:, :, None])).sum(-1)
        return loc @ self.phi.T                                             # [E, nq]


def helium(m, p, Z=2.0, n_occ=2.0, n_states=4, n_guard=2, mixing=0.3, max_iter=60, tol=1e-9, rc=0.05, seed=7):
    m = ks.meshmod.mark_all_boundary(m)
    S = oracle.Space(m, p, quad_q=p + 2)
    K0 = S.assemble("stiff")
    K = K0.copy()
    S.zero_bc(K, None, 1)
    M = S.assemble("mass")
    S.zero_bc(M, None, 1)
    Ks = _to_scipy(K)
    q = S.element_qpoints()
    W = S.geometry()["volume"][:, None] * S.quadrature()["w3"][None, :]
    vext = ks._v_ext(np.linalg.norm(q, axis=-1), Z, rc)
    ev = _Eval(S)
    n = S.n_dof
    k = n_states + n_guard
    X = np.random.default_rng(seed).uniform(-1.0, 1.0, (k, n))
    for j in range(k):
        c = np.ascontiguousarray(X[j])
        S.zero_bc(None, c, 1)
        X[j] = c
    c_x = float(np.cbrt(3.0 / np.pi))
    rho = np.zeros_like(vext)
    vh = np.zeros_like(vext)
    E_old = np.inf
    dE = np.inf
    P = oracle.PMG(K, p, S.sum_dof(), 2)
    for it in range(1, max_iter + 1):
        cr = np.cbrt(rho)
        vx = -c_x * cr
        H = _to_scipy(S.assemble_potential(vext + vh + vx)) + 0.5 * Ks
        Hc = _from_scipy(H)
        S.zero_bc(Hc, None, 1)
        # eigenpairs as accurate as the density deserves, 1e-10 at the end
        etol = 1e-3 if it == 1 else max(1e-10, min(1e-4, 1e-2 * abs(dE)))
        lam, X, st = oracle.lobpcg(Hc, M, X, tol=etol, max_it=2000, precond=4, pmg=P, smooth=2)
        e_h = 0.5 * float(np.sum(W * vh * rho))
        e_xc = float(np.sum(W * (-0.75 * c_x * cr ** 4 - vx * rho)))
        E = n_occ * float(lam[0]) - e_h + e_xc
        dE = E - E_old if np.isfinite(E_old) else np.inf
        if abs(dE) < tol and etol <= 1e-10:
            return E, lam[:n_states], it
        E_old = E
        rho_out = S.density(X[:1], [n_occ])
        rho = rho_out if it == 1 else rho + mixing * (rho_out - rho)
        mom = ks.multipole_moments(W, q, rho)
        frho = 4.0 * np.pi * rho
        b = S.rhs(lambda pts: frho)
        # as SCFIteration.cpp:170-176: a fresh copy of the stiffness matrix, the boundary
        # data imposed on it with the matrix modified, PCG on the copy
        Kh = K0.copy()
        S.dirichlet(Kh, b, lambda pts: ks.multipole_potential(mom, pts), True, 1)
        vh_dofs, _ = oracle.pcg(Kh, b, tol=0.0, rel_tol=1e-13, max_step=20000, flag=1)
        vh = ev(vh_dofs)
    raise RuntimeError("oracle SCF did not converge")
