"""Generate the oracle's answers at the benchmark configurations as small fixtures.

The oracle (the CPU restatement of TSEMLib's FP64 path) is run once here at sizes
that take it minutes, and only what the GPU tests compare against is kept:

  poisson_N24_p6.npz  unit-cube Poisson, mixed boundary conditions, N = 24 Kuhn
                      sub-cubes per side, jitter 0.1 h (seed 2024), p = 6, quadrature
                      q = 8 (3 048 625 DOFs); p-multigrid PCG (orders 6-4-2-1, two
                      Gauss-Seidel sweeps): iterations to relative residual 1e-10 and
                      to 1e-12, the 1e-12 solution at 8192 seeded DOFs, its sum, sum
                      of squares, L2 and H1 errors, and a checksum of the mesh.
  laplace_N16_p5_k20.npz
                      Dirichlet Laplace eigenpairs, N = 16, no jitter, p = 5,
                      quadrature q = 7 (531 441 DOFs); the oracle's block LOBPCG with
                      k = 20 from the seeded block U(-1, 1) (seed 2024), p-multigrid
                      preconditioner, residual tolerance 1e-10: the 20 eigenvalues.

    python tests/golden/make_config_fixtures.py [poisson|laplace|all]

The GPU tests (tests/test_gpu_config_parity.py) rebuild the same meshes and compare.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from tsemlib_gb300 import manufactured as mf  # noqa: E402
from tsemlib_gb300 import mesh  # noqa: E402

SAMPLES = 8192


def poisson(n=24, p=6, seed=2024):
    m = mesh.mark_box_boundary(mesh.kuhn_cube(n, 0.1, seed), [(0, 0.0), (0, 1.0)])
    t0 = time.time()
    S = oracle.Space(m, p, quad_q=p + 2)
    A = S.assemble("stiff")
    b = S.rhs(mf.f_cfg1)
    S.neumann(b, mf.neumann_cfg1, 2)
    S.dirichlet(A, b, mf.u_cfg1, True, 1)
    P = oracle.PMG(A, p, S.sum_dof(), 2)
    print(f"poisson N={n} p={p}: n={A.n} nnz={A.nnz} setup {time.time() - t0:.1f} s", flush=True)
    t0 = time.time()
    _, s10 = oracle.pcg(A, b, tol=0.0, rel_tol=1e-10, max_step=5000, flag=4, pmg=P, smooth=2)
    t10 = time.time() - t0
    print(f"  to 1e-10: {s10['iterations']} iterations, {t10:.1f} s", flush=True)
    t0 = time.time()
    x, s12 = oracle.pcg(A, b, tol=0.0, rel_tol=1e-12, max_step=5000, flag=4, pmg=P, smooth=2)
    print(f"  to 1e-12: {s12['iterations']} iterations, {time.time() - t0:.1f} s", flush=True)
    l2, h1 = S.errors(x, mf.u_cfg1, mf.grad_cfg1)
    idx = np.sort(np.random.default_rng(7).choice(A.n, SAMPLES, replace=False))
    out = os.path.join(HERE, f"poisson_N{n}_p{p}.npz")
    np.savez_compressed(out, n=n, p=p, seed=seed, n_dof=A.n, nnz=A.nnz, xyz_sum=float(m.xyz.sum()),
                        iterations_1e10=s10["iterations"], iterations_1e12=s12["iterations"],
                        seconds_1e10=t10, threads=oracle.get_threads(),
                        idx=idx, x=x[idx], x_sum=float(x.sum()), x_sq=float(x @ x), l2=l2, h1=h1)
    print("wrote", out, flush=True)


def laplace(n=16, p=5, k=20, seed=2024):
    m = mesh.mark_all_boundary(mesh.kuhn_cube(n, 0.0, 1))
    t0 = time.time()
    S = oracle.Space(m, p, quad_q=p + 2)
    A = S.assemble("stiff")
    M = S.assemble("mass")
    S.zero_bc(A, None, 1)
    S.zero_bc(M, None, 1)
    P = oracle.PMG(A, p, S.sum_dof(), 2)
    X0 = np.random.default_rng(seed).uniform(-1.0, 1.0, (A.n, k))
    for j in range(k):
        c = np.ascontiguousarray(X0[:, j])
        S.zero_bc(None, c, 1)
        X0[:, j] = c
    print(f"laplace N={n} p={p}: n={A.n} setup {time.time() - t0:.1f} s", flush=True)
    t0 = time.time()
    lam, _, st = oracle.lobpcg(A, M, np.ascontiguousarray(X0.T), tol=1e-10, max_it=500, precond=4, pmg=P, smooth=2)
    print(f"  LOBPCG: {st}, {time.time() - t0:.1f} s", flush=True)
    out = os.path.join(HERE, f"laplace_N{n}_p{p}_k{k}.npz")
    np.savez_compressed(out, n=n, p=p, k=k, seed=seed, n_dof=A.n, xyz_sum=float(m.xyz.sum()), lam=lam,
                        iterations=st["iterations"], residual=st["residual"], status=st["status"])
    print("wrote", out, lam[:16], flush=True)


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    oracle.build()
    if what in ("poisson", "all"):
        poisson()
    if what in ("laplace", "all"):
        laplace()
