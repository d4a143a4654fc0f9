"""Kohn-Sham self-consistent field for a helium-like atom (TSEMLib's
examples/KohnSham-Helium/SCFIteration.cpp) on the GPU library.

Domain [-L, L]^3 with a Kuhn mesh graded geometrically towards the nucleus at the
origin, order p, zero Dirichlet conditions.  Every SCF step:

* effective potential at the element quadrature points,
  V = V_ext + V_H + V_x, V_ext = -Z/r (smoothed inside r_c by the quadratic that
  matches value and slope), V_x = -(3 rho / pi)^(1/3) (LDA exchange,
  SCFIteration.cpp:224);
* Hamiltonian H = K / 2 + M_V (build_mass_V_matrix, src/Discretize.cpp:668-843);
* block LOBPCG for the lowest states, preconditioned by the matrix-free p-multigrid
  V-cycle of K (SCFIteration.cpp:397);
* density rho = occ |psi_0|^2 mixed linearly into the previous one, kinetic energy
  mixed alike (SCFIteration.cpp:53-67);
* Hartree potential from -Lap V_H = 4 pi rho with V_H on the boundary from the
  density's multipole expansion to quadrupole order (SCFIteration.cpp:70-153),
  solved with the mixed solver;
* energy of the input density, occ eps_0 - E_H + int (eps_x - V_x) rho (the
  Kohn-Sham energy at self-consistency, SCFIteration.cpp:228-257; written with the
  band energy its error is second order in the density error), stop when it changes
  by less than tol with the eigenpairs at eig_tol.

LDA correlation (VWN, SCFIteration.cpp:192-223) is not included: the workload
asks for exchange only.

The [E, nq] point arrays (potential, density, Hartree potential) stay in GPU memory
as FP64 torch tensors; the library's device-array calls evaluate FE functions at
the points, assemble M_V and form right-hand sides from them.  The Hartree
boundary values are imposed on the right-hand side against the unmodified
stiffness matrix (the solver already holds the eliminated one).
"""
from __future__ import annotations

import time

import numpy as np

from . import mesh as meshmod
from . import tsem


def multipole_moments(W, q, rho):
    """The ten moments of the density that the Hartree boundary data uses
    (SCFIteration.cpp:70-97): int rho, int x_i rho, int x_i x_j rho (i <= j, in the
    order xx, xy, xz, yy, yz, zz).  W [E, nq] integration weights, q [E, nq, 3]
    quadrature points, rho [E, nq]; any array library with broadcasting and sum."""
    x, y, z = q[..., 0], q[..., 1], q[..., 2]
    wr = W * rho
    comps = [1.0, x, y, z, x * x, x * y, x * z, y * y, y * z, z * z]
    return [float((wr * c).sum()) for c in comps]


def multipole_potential(c, pts):
    """Hartree potential of a density with moments c (multipole_moments) at points far
    from it, to quadrupole order, term by term as calc_multipole_expansion
    (SCFIteration.cpp:98-115) writes it: Q / r + p . r^ / r^2 + 1/2 sum_i c_ii
    (3 x^_i^2 - 1) / r^3 + 3 sum_{i<j} c_ij x^_i x^_j / r^3."""
    x, y, z = pts[..., 0], pts[..., 1], pts[..., 2]
    r = np.sqrt(x * x + y * y + z * z)
    # points near the charge (where the expansion does not hold; callers sample every
    # geometry and keep the boundary ones) give large or non-finite values
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        ir = 1.0 / np.maximum(r, 1e-300)
        xr, yr, zr = x * ir, y * ir, z * ir
        return (c[0] * ir + (c[1] * xr + c[2] * yr + c[3] * zr) * ir ** 2
                + 0.5 * (c[4] * (3 * xr * xr - 1) + c[7] * (3 * yr * yr - 1) + c[9] * (3 * zr * zr - 1)) * ir ** 3
                + 3.0 * (c[5] * xr * yr + c[6] * xr * zr + c[8] * yr * zr) * ir ** 3)


def _v_ext(r, Z, rc):
    out = np.empty_like(r)
    far = r >= rc
    out[far] = -Z / r[far]
    x = r[~far] / rc
    out[~far] = -Z / rc * (1.5 - 0.5 * x * x)
    return out


def helium(p=5, n_half=10, ratio=1.15, half_width=10.0, Z=2.0, n_occ=2.0, n_states=4, n_guard=2, mixing=0.3,
           max_iter=40, tol=1e-8, rc=0.05, eig_tol=1e-8, seed=7, mesh_in=None):
    """mesh_in: a mesh to run on instead of the graded Kuhn cube (for instance the
    reference's cube_atom.mesh through mesh.read_afepack); its whole boundary gets the
    zero Dirichlet condition."""
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    t0 = time.perf_counter()
    if mesh_in is not None:
        m = meshmod.mark_all_boundary(mesh_in)
    else:
        coords = meshmod.graded_coords(n_half, ratio, half_width)
        m = meshmod.mark_all_boundary(meshmod.kuhn_cube(len(coords) - 1, 0.0, 0, coords=coords))
    T = tsem.TSEM(p, p + 2, m)
    K = T.stiff_matrix.copy()
    T.impose_zero_boundary_condition(K, None, 1)
    M = T.mass_matrix.copy()
    T.impose_zero_boundary_condition(M, None, 1)
    mx = tsem.MixedSolver(T, K, 1, order_step=2, tol_rel=1e-12)
    q = T.element_qpoints()
    r = np.linalg.norm(q, axis=-1)
    W_h = T.geometry()["volume"][:, None] * T.quadrature()["w3"][None, :]    # integration weights [E, nq]
    W = torch.from_numpy(W_h).to(dev)
    vext = torch.from_numpy(_v_ext(r, Z, rc)).to(dev)
    qd = torch.from_numpy(q).to(dev)
    n = T.n_dof_total

    def at_points(x_host):
        """[E, nq] device values of the FE function with coefficients x_host"""
        xd = torch.from_numpy(np.ascontiguousarray(x_host, dtype=np.float64)).to(dev)
        out = torch.empty_like(vext)
        T.value_qp_device(xd.data_ptr(), out.data_ptr(), sh)
        return out
    k = n_states + n_guard
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1.0, 1.0, (n, k)) * np.exp(-np.linalg.norm(_dof_points_guess(T, n), axis=-1))[:, None]
    for j in range(k):
        col = np.ascontiguousarray(X[:, j])
        T.impose_zero_boundary_condition(None, col, 1)
        X[:, j] = col
    setup_s = time.perf_counter() - t0

    rho = torch.zeros_like(vext)    # input density of the step (bare nucleus first)
    vh = torch.zeros_like(vext)     # Hartree potential of rho
    c_x = float(np.cbrt(3.0 / np.pi))
    E_old = np.inf
    H = None
    history = []
    lam = None
    converged = False
    t1 = time.perf_counter()
    for it in range(1, max_iter + 1):
        ta = time.perf_counter()
        cr = torch.pow(rho, 1.0 / 3.0)
        vx = -c_x * cr
        V = (vext + vh + vx).contiguous()
        H = T.build_mass_V_matrix_device(V.data_ptr(), out=H, stream=sh)
        H.add(0.5, K)
        T.impose_zero_boundary_condition(H, None, 1)
        tb = time.perf_counter()
        # eigenpairs only as accurate as the density deserves: loose while the
        # energy still moves, eig_tol at the end
        etol = 1e-3 if it == 1 else max(eig_tol, min(1e-4, 1e-2 * abs(dE)))
        lam, st = mx.solve_LOBPCG(X, M, tol=etol, max_step=500, n_want=n_states, A=H)
        tc = time.perf_counter()
        # energy of the input density (band energy minus double counting; its error is
        # second order in the density error, so it settles faster than the density)
        e_h = 0.5 * float(torch.sum(W * vh * rho))
        e_xc = float(torch.sum(W * (-0.75 * c_x * cr ** 4 - vx * rho)))
        E = n_occ * float(lam[0]) - e_h + e_xc
        Q = float(torch.sum(W * rho))
        history.append(dict(iteration=it, energy=E, eigenvalues=lam[:n_states].tolist(), lobpcg_iterations=st["iterations"],
                            lobpcg_tol=etol, charge=Q, hamiltonian_s=tb - ta, lobpcg_s=tc - tb))
        dE = E - E_old if np.isfinite(E_old) else np.inf
        if abs(dE) < tol and etol <= eig_tol:
            converged = True
            break
        E_old = E
        # output density, linear mixing, Hartree potential of the mixed density
        psi = torch.from_numpy(np.ascontiguousarray(X[:, 0])).to(dev)
        rho_out = torch.empty_like(vext)
        T.calc_density_device(psi.data_ptr(), [n_occ], rho_out.data_ptr(), sh)     # SCFIteration.cpp:63
        rho = rho_out if it == 1 else rho + mixing * (rho_out - rho)
        moments = multipole_moments(W, qd, rho)
        td = time.perf_counter()
        f = (4.0 * np.pi * rho).contiguous()
        b_d = torch.empty(n, dtype=torch.float64, device=dev)
        T.calc_rhs_device(f.data_ptr(), b_d.data_ptr(), sh)
        b = b_d.cpu().numpy()
        # V_H on the boundary from the density's multipole expansion: right-hand side of
        # the eliminated system, formed against the unmodified stiffness matrix (the
        # right-hand side SCFIteration.cpp:170-172 gets by imposing on a fresh copy with
        # the matrix modified, without the copy)
        T.impose_boundary_condition(T.stiff_matrix, b, lambda pts: multipole_potential(moments, pts), False, 1)
        te = time.perf_counter()
        history[-1]["moments"] = moments
        vh_dofs = np.zeros(n)
        st_h = mx.solve(vh_dofs, b)
        tf = time.perf_counter()
        vh = at_points(vh_dofs)
        tg = time.perf_counter()
        history[-1].update(density_hartree_s=tg - tc, density_moments_s=td - tc, rhs_boundary_s=te - td,
                           hartree_solve_s=tf - te, hartree_points_s=tg - tf, hartree_iterations=st_h["iterations"])
    scf_s = time.perf_counter() - t1
    return dict(energy=E, eigenvalues=lam[:n_states].tolist(), iterations=len(history), converged=converged,
                n_dof=n, history=history, setup_s=setup_s, scf_s=scf_s)


def _dof_points_guess(T, n):
    """A point per DOF for shaping the initial block: the mean of the quadrature
    points of the elements, spread over the DOFs they touch (decays away from the
    nucleus, so the start is not dominated by the boundary layer)."""
    tn, ti, tv = T.transform()
    q = T.element_qpoints().mean(axis=1)                       # [E, 3]
    acc = np.zeros((n, 3))
    cnt = np.zeros(n)
    idx = ti[:, :, 0]
    valid = idx >= 0
    e_of = np.broadcast_to(np.arange(idx.shape[0])[:, None], idx.shape)
    np.add.at(acc, idx[valid], q[e_of[valid]])
    np.add.at(cnt, idx[valid], 1.0)
    return acc / np.maximum(cnt, 1.0)[:, None]
