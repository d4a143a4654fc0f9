"""Manufactured solution of the unit-cube Poisson workloads (u = sin(pi x) sin(pi y)
sin(pi z) + x^2 with Dirichlet data on x = 0, 1 and Neumann data elsewhere): u, its
gradient, the source f = -Laplace u and the outward normal derivative on the faces
y = 0, 1 and z = 0, 1.  Shared by the benchmark, the smoke check and the tests."""
import numpy as np

PI = np.pi


def u_cfg1(p):
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    return np.sin(PI * x) * np.sin(PI * y) * np.sin(PI * z) + x * x


def f_cfg1(p):
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    return 3 * PI * PI * np.sin(PI * x) * np.sin(PI * y) * np.sin(PI * z) - 2


def grad_cfg1(p):
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    return np.stack([PI * np.cos(PI * x) * np.sin(PI * y) * np.sin(PI * z) + 2 * x,
                     PI * np.sin(PI * x) * np.cos(PI * y) * np.sin(PI * z),
                     PI * np.sin(PI * x) * np.sin(PI * y) * np.cos(PI * z)], -1)


def neumann_cfg1(p, tol=1e-12):
    """Outward normal derivative of u_cfg1 on the faces y = 0, 1 and z = 0, 1."""
    y, z = p[..., 1], p[..., 2]
    g = grad_cfg1(p)
    out = np.zeros(p.shape[:-1])
    out = np.where(np.abs(y) < tol, -g[..., 1], out)
    out = np.where(np.abs(y - 1) < tol, g[..., 1], out)
    out = np.where(np.abs(z) < tol, -g[..., 2], out)
    out = np.where(np.abs(z - 1) < tol, g[..., 2], out)
    return out
