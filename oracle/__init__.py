"""TEST INFRASTRUCTURE ONLY -- ctypes binding of the CPU oracle.

The oracle is a plain FP64 C++ restatement of TSEMLib's discretise-and-solve path
(see oracle/oracle.hpp).  Only tests/, ``__graft_entry__.smoke()`` and the CPU
baseline leg of bench.py use it, and only as the checker or the timed CPU
reference; the shipped library never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboracle_tsem.so")
FACE_TABLE = os.path.join(os.path.dirname(_HERE), "tests", "golden", "face_table_M10.txt")

_lib = None

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_L = ctypes.c_int64


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, a few seconds; make rebuilds only
    when a source is newer than the library)."""
    subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return LIB_PATH


def build_ref() -> None:
    """Build oracle/_ref/ from the parts of TSEMLib that compile on their own (the
    multi-index headers), where the reference tree is present; otherwise a no-op."""
    subprocess.run(["make", "-s", "-C", _HERE, "ref"], check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        sig = {
            "or_last_error": (ctypes.c_char_p, []),
            "or_set_threads": (None, [_I]),
            "or_get_threads": (_I, []),
            "or_space_create": (_P, [_I, _P, _I, _P, _I, _P, _P, _I, _P, _P, _P, _P, _P, _P, _P, _I, ctypes.c_char_p, _I]),
            "or_space_free": (None, [_P]),
            "or_space_info": (None, [_P, _P]),
            "or_space_geometry": (None, [_P] * 10),
            "or_space_numbering": (None, [_P, _P, _P]),
            "or_space_transform": (None, [_P, _P, _P, _P]),
            "or_multiindex": (None, [_I, _P, _P]),
            "or_sum_dof": (None, [_P, _P]),
            "or_refmat": (_I, [_P, _I, _I, _P, _P]),
            "or_basis_values": (None, [_P, _P, _P]),
            "or_basis_gradients": (None, [_P, _P, _P]),
            "or_jacobi_values": (None, [_P, _P, _P]),
            "or_quadrature": (None, [_P] * 7),
            "or_element_qpoints": (None, [_P, _P]),
            "or_boundary_points": (_L, [_P, _I, _P]),
            "or_rhs": (None, [_P, _P, _P]),
            "or_assemble_potential": (_P, [_P, _P]),
            "or_errors": (None, [_P, _P, _P, _P, _P]),
            "or_density": (None, [_P, _P, _I, _P, _P]),
            "or_density_l2_difference": (_D, [_P, _P, _P, _I, _P]),
            "or_assemble": (_P, [_P, _I]),
            "or_csr_import": (_P, [_I, _P, _P, _P]),
            "or_csr_copy": (_P, [_P]),
            "or_csr_free": (None, [_P]),
            "or_csr_nnz": (_L, [_P]),
            "or_csr_n": (_I, [_P]),
            "or_csr_export": (None, [_P, _P, _P, _P]),
            "or_csr_vmult": (None, [_P, _P, _P]),
            "or_dirichlet": (_I, [_P, _P, _P, _P, _P, _P, _I, _I]),
            "or_neumann": (_I, [_P, _P, _P, _I]),
            "or_zero_bc": (_I, [_P, _P, _P, _I]),
            "or_interpolation": (_I, [_P, _P, _P, _P, _P, _P]),
            "or_space_set_quadrature": (_I, [_P, _I, _P, _P, _I, _P, _P, _I, _P, _P]),
            "or_pmg_create": (_P, [_P, _I, _P, _I]),
            "or_pmg_free": (None, [_P]),
            "or_pmg_levels": (_I, [_P, _P]),
            "or_pmg_level_matrix": (_P, [_P, _I]),
            "or_pmg_core_at": (None, [_P, _I, _P]),
            "or_pmg_vcycle": (None, [_P, _P, _P, _I]),
            "or_gs": (None, [_P, _P, _P, _I, _I]),
            "or_pcg": (_I, [_P, _P, _P, _D, _D, _I, _I, _P, _I, _D, _P]),
            "or_inverse_power": (_D, [_P, _P, _P, _D, _I, _P]),
            "or_lobpcg": (_I, [_P, _P, _I, _P, _P, _D, _I, _I, _P, _I, _P]),
            "or_sym_eig": (None, [_I, _P, _P, _P]),
            "or_rayleigh_ritz": (_I, [_I, _P, _P, _P, _P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def multiindex(M: int):
    """The oracle's multi-index table of order M: [n][3] multi-indices by number,
    and the number of each back again."""
    n = (M + 1) * (M + 2) * (M + 3) // 6
    alpha = np.empty((n, 3), np.int32)
    number = np.empty(n, np.int32)
    lib().or_multiindex(M, _ptr(alpha), _ptr(number))
    return alpha, number


def set_threads(n: int) -> None:
    """Number of OpenMP threads the oracle's parallel loops use from now on."""
    lib().or_set_threads(int(n))


def get_threads() -> int:
    return lib().or_get_threads()


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Csr:
    """Owned handle to an oracle CSR matrix (diagonal first in every row)."""

    def __init__(self, handle):
        if not handle:
            raise RuntimeError(lib().or_last_error().decode())
        self.h = handle

    @classmethod
    def from_arrays(cls, rowptr, col, val):
        rowptr = _c(rowptr, np.int64); col = _c(col, np.int32); val = _c(val, np.float64)
        return cls(lib().or_csr_import(len(rowptr) - 1, _ptr(rowptr), _ptr(col), _ptr(val)))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.or_csr_free(self.h)
            self.h = None

    def copy(self):
        return Csr(lib().or_csr_copy(self.h))

    @property
    def n(self):
        return lib().or_csr_n(self.h)

    @property
    def nnz(self):
        return lib().or_csr_nnz(self.h)

    def arrays(self):
        n, nnz = self.n, self.nnz
        rp = np.empty(n + 1, np.int64); c = np.empty(nnz, np.int32); v = np.empty(nnz, np.float64)
        lib().or_csr_export(self.h, _ptr(rp), _ptr(c), _ptr(v))
        return rp, c, v

    def matvec(self, x):
        x = _c(x, np.float64)
        y = np.empty(self.n)
        lib().or_csr_vmult(self.h, _ptr(x), _ptr(y))
        return y


class PMG:
    def __init__(self, A: Csr, p: int, sum_dof, step: int = 1):
        s = _c(sum_dof, np.int32)
        self.A = A
        self.h = lib().or_pmg_create(A.h, p, _ptr(s), step)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.or_pmg_free(self.h)
            self.h = None

    def levels(self):
        n = lib().or_pmg_levels(self.h, None)
        out = np.empty(n + 1, np.int32)
        lib().or_pmg_levels(self.h, _ptr(out))
        return out

    def level_arrays(self, level):
        h = lib().or_pmg_level_matrix(self.h, level)
        n, nnz = lib().or_csr_n(h), lib().or_csr_nnz(h)
        rp = np.empty(n + 1, np.int64); c = np.empty(nnz, np.int32); v = np.empty(nnz, np.float64)
        lib().or_csr_export(h, _ptr(rp), _ptr(c), _ptr(v))
        return rp, c, v

    def core_at(self, level):
        lv = self.levels()
        out = np.empty(lv[level], np.int32)
        lib().or_pmg_core_at(self.h, level, _ptr(out))
        return out

    def vcycle(self, r, x=None, smooth=2):
        r = _c(r, np.float64)
        x = np.zeros_like(r) if x is None else _c(x, np.float64).copy()
        lib().or_pmg_vcycle(self.h, _ptr(x), _ptr(r), smooth)
        return x


class Space:
    """The oracle's TSEM space on an AFEPack-style mesh (tsemlib_gb300.mesh.TetMesh)."""

    def __init__(self, mesh, p: int, quad_q: int = 10, face_table: str = FACE_TABLE):
        L = lib()
        self.mesh = mesh
        self.p = p
        m = mesh
        self._keep = [_c(m.xyz, np.float64), _c(m.edge_v, np.int32), _c(m.face_v, np.int32), _c(m.face_e, np.int32),
                      _c(m.tet_v, np.int32), _c(m.tet_f, np.int32), _c(m.mark_v, np.int32), _c(m.mark_e, np.int32),
                      _c(m.mark_f, np.int32), _c(m.femdof_v, np.int32), _c(m.femdof_e, np.int32)]
        k = self._keep
        self.h = L.or_space_create(m.nv, _ptr(k[0]), m.ne, _ptr(k[1]), m.nf, _ptr(k[2]), _ptr(k[3]), m.nt, _ptr(k[4]),
                                   _ptr(k[5]), _ptr(k[6]), _ptr(k[7]), _ptr(k[8]), _ptr(k[9]), _ptr(k[10]), p,
                                   face_table.encode(), quad_q)
        if not self.h:
            raise RuntimeError(L.or_last_error().decode())
        info = np.zeros(16, np.int32)
        L.or_space_info(self.h, _ptr(info))
        (self.n_dof, self.n_loc, self.max_dep, self.n_ele, self.nq3, self.nq2, self.nq1) = [int(x) for x in info[:7]]
        self.n_geo = [int(x) for x in info[7:11]]
        self.n_dof_geo = [int(x) for x in info[11:15]]

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.or_space_free(self.h)
            self.h = None

    # ---- structure
    def geometry(self):
        m = self.mesh
        E = self.n_ele
        out = dict(type_edge=np.empty(6 * E, np.int32), type_face=np.empty(4 * E, np.int32),
                   type_face_inv=np.empty(4 * E, np.int32), edge_node=np.empty(2 * m.ne, np.int32),
                   face_node=np.empty(3 * m.nf, np.int32), face_edge=np.empty(3 * m.nf, np.int32),
                   face_same=np.empty(3 * m.nf, np.uint8), volume=np.empty(E), ele_edge=np.empty(6 * E, np.int32))
        lib().or_space_geometry(self.h, *[_ptr(out[k]) for k in ["type_edge", "type_face", "type_face_inv", "edge_node",
                                                                 "face_node", "face_edge", "face_same", "volume",
                                                                 "ele_edge"]])
        return out

    def numbering(self):
        ng = sum(self.n_geo)
        lg = np.empty(ng, np.int32); la = np.empty(ng, np.int32)
        lib().or_space_numbering(self.h, _ptr(lg), _ptr(la))
        return lg, la

    def transform(self):
        E, nl, md = self.n_ele, self.n_loc, self.max_dep
        tn = np.empty(E * nl, np.int32); ti = np.empty(E * nl * md, np.int32); tv = np.empty(E * nl * md)
        lib().or_space_transform(self.h, _ptr(tn), _ptr(ti), _ptr(tv))
        return tn.reshape(E, nl), ti.reshape(E, nl, md), tv.reshape(E, nl, md)

    def sum_dof(self):
        out = np.empty(self.n_dof, np.int32)
        lib().or_sum_dof(self.h, _ptr(out))
        return out

    def refmat(self, which: int, actual: bool = True):
        n = lib().or_refmat(self.h, which, int(actual), None, None)
        d = np.empty((n, n)); pat = np.empty((n, n), np.uint8)
        lib().or_refmat(self.h, which, int(actual), _ptr(d), _ptr(pat))
        return d, pat.astype(bool)

    def basis_values(self, pt):
        pt = _c(pt, np.float64); out = np.empty(self.n_loc)
        lib().or_basis_values(self.h, _ptr(pt), _ptr(out))
        return out

    def basis_gradients(self, pt):
        pt = _c(pt, np.float64); out = np.empty((self.n_loc, 3))
        lib().or_basis_gradients(self.h, _ptr(pt), _ptr(out))
        return out

    def quadrature(self):
        x3 = np.empty((self.nq3, 3)); w3 = np.empty(self.nq3); b2 = np.empty((self.nq2, 3)); w2 = np.empty(self.nq2)
        x1 = np.empty(self.nq1); w1 = np.empty(self.nq1)
        lib().or_quadrature(self.h, *[_ptr(a) for a in (x3, w3, b2, w2, x1, w1)])
        return dict(x3=x3, w3=w3, b2=b2, w2=w2, x1=x1, w1=w1)

    def element_qpoints(self):
        out = np.empty((self.n_ele, self.nq3, 3))
        lib().or_element_qpoints(self.h, _ptr(out))
        return out

    def boundary_points(self, dim):
        n = lib().or_boundary_points(self.h, dim, None)
        out = np.empty((n, 3))
        lib().or_boundary_points(self.h, dim, _ptr(out))
        return out

    # ---- discretisation
    def assemble(self, which: str) -> Csr:
        return Csr(lib().or_assemble(self.h, 0 if which == "stiff" else 1))

    def assemble_potential(self, v_qp):
        """build_mass_V_matrix with V at the element quadrature points ([E, nq])."""
        v = _c(v_qp, np.float64)
        return Csr(lib().or_assemble_potential(self.h, _ptr(v)))

    def rhs(self, f):
        """f: callable on [..., 3] points -> values."""
        fq = _c(f(self.element_qpoints()), np.float64)
        out = np.empty(self.n_dof)
        lib().or_rhs(self.h, _ptr(fq), _ptr(out))
        return out

    def dirichlet(self, A: Csr, rhs, u, modify=True, flag=1):
        vb = [_c(u(self.boundary_points(d)), np.float64) for d in range(3)]
        r = lib().or_dirichlet(self.h, A.h, _ptr(rhs), _ptr(vb[0]), _ptr(vb[1]), _ptr(vb[2]), int(modify), flag)
        if r != 0:
            raise RuntimeError(lib().or_last_error().decode())

    def neumann(self, rhs, g, flag=2):
        g2 = _c(g(self.boundary_points(2)), np.float64)
        if lib().or_neumann(self.h, _ptr(rhs), _ptr(g2), flag) != 0:
            raise RuntimeError(lib().or_last_error().decode())

    def set_quadrature(self, x1, w1, b2, w2, x3, w3):
        """read_quad_info (src/QuadInfo.cpp:13-60): a tabulated rule in place of the
        collapsed Gauss rule (x1 [n1] in [0, 1], b2 [n2, 3], x3 [n3, 3], unit weights)."""
        a = [_c(v, np.float64) for v in (x1, w1, b2, w2, x3, w3)]
        self._rule = a
        if lib().or_space_set_quadrature(self.h, len(a[1]), _ptr(a[0]), _ptr(a[1]), len(a[3]), _ptr(a[2]),
                                         _ptr(a[3]), len(a[5]), _ptr(a[4]), _ptr(a[5])) != 0:
            raise RuntimeError(lib().or_last_error().decode())
        self.nq1, self.nq2, self.nq3 = len(a[1]), len(a[3]), len(a[5])

    def interpolation(self, u):
        """calc_interpolation (src/Interpolation.cpp:12-101) of the function u, sampled at
        every vertex, edge and face point and at the element quadrature points."""
        vb = [_c(u(self.boundary_points(d)), np.float64) for d in range(3)]
        uq = _c(u(self.element_qpoints()), np.float64)
        out = np.empty(len(self.sum_dof()))
        if lib().or_interpolation(self.h, _ptr(vb[0]), _ptr(vb[1]), _ptr(vb[2]), _ptr(uq), _ptr(out)) != 0:
            raise RuntimeError(lib().or_last_error().decode())
        return out

    def zero_bc(self, A: Csr | None, rhs=None, flag=1):
        if lib().or_zero_bc(self.h, None if A is None else A.h, _ptr(rhs), flag) != 0:
            raise RuntimeError(lib().or_last_error().decode())

    def errors(self, sol, u, grad_u):
        q = self.element_qpoints()
        uq = _c(u(q), np.float64); gq = _c(grad_u(q), np.float64)
        sol = _c(sol, np.float64)
        out = np.empty(2)
        lib().or_errors(self.h, _ptr(sol), _ptr(uq), _ptr(gq), _ptr(out))
        return float(out[0]), float(out[1])

    def density(self, states, occ):
        """calc_density (src/PointInfo.cpp:72-91): sum_j occ_j psi_j^2 at the element
        quadrature points [E, nq]; states [k, n_dof]"""
        st = _c(np.atleast_2d(states), np.float64)
        oc = _c(occ, np.float64)
        out = np.empty((self.n_ele, self.nq3))
        lib().or_density(self.h, _ptr(st), st.shape[0], _ptr(oc), _ptr(out))
        return out

    def density_l2_difference(self, u, v, occ):
        """calc_density_l2_difference (src/CalcError.cpp:703-735); u, v [k, n_dof]"""
        u = _c(np.atleast_2d(u), np.float64); v = _c(np.atleast_2d(v), np.float64)
        oc = _c(occ, np.float64)
        return float(lib().or_density_l2_difference(self.h, _ptr(u), _ptr(v), u.shape[0], _ptr(oc)))


def pcg(A: Csr, b, x0=None, tol=1e-14, rel_tol=0.0, max_step=100000, flag=1, pmg: PMG | None = None, smooth=2,
        omega=1.0):
    """Reference PCG (src/TSEMSolver.cpp:1776-1929).  flags 2 / 3 (SOR / SSOR) use omega
    and `smooth` sweeps.  Returns (x, stats dict)."""
    b = _c(b, np.float64)
    x = np.zeros_like(b) if x0 is None else _c(x0, np.float64).copy()
    st = np.zeros(5)
    it = lib().or_pcg(A.h, _ptr(x), _ptr(b), tol, rel_tol, max_step, flag, None if pmg is None else pmg.h, smooth,
                      float(omega), _ptr(st))
    if it < 0:
        raise RuntimeError(lib().or_last_error().decode())
    return x, dict(iterations=int(st[0]), residual_l1=st[1], init_l1=st[2], residual_l2=st[3], status=int(st[4]))


def gs(A: Csr, x, r, steps=1, direction=0):
    x = _c(x, np.float64).copy(); r = _c(r, np.float64)
    lib().or_gs(A.h, _ptr(x), _ptr(r), steps, direction)
    return x


def inverse_power(A: Csr, B: Csr, x0, tol=1e-10, max_step=1000):
    x = _c(x0, np.float64).copy()
    it = ctypes.c_int(0)
    e = lib().or_inverse_power(A.h, B.h, _ptr(x), tol, max_step, ctypes.byref(it))
    return e, x, it.value


def lobpcg(A: Csr, B: Csr, X0, tol=1e-8, max_it=500, precond=4, pmg: PMG | None = None, smooth=2):
    """Block LOBPCG; X0 is [k, n].  Returns (lambda, X, stats)."""
    X = _c(X0, np.float64).copy()
    k = X.shape[0]
    lam = np.empty(k); st = np.zeros(3)
    r = lib().or_lobpcg(A.h, B.h, k, _ptr(X), _ptr(lam), tol, max_it, precond, None if pmg is None else pmg.h, smooth,
                        _ptr(st))
    if r < 0:
        raise RuntimeError(lib().or_last_error().decode())
    return lam, X, dict(iterations=int(st[0]), residual=st[1], status=int(st[2]))


def sym_eig(a):
    a = _c(a, np.float64); n = a.shape[0]
    w = np.empty(n); v = np.empty((n, n))
    lib().or_sym_eig(n, _ptr(a), _ptr(w), _ptr(v))
    return w, v


def rayleigh_ritz(ga, gb):
    """The oracle's Rayleigh-Ritz step of its LOBPCG (the generalised eigensolve the
    reference hands to LAPACKE_dsygvx): Ritz values of the numerically independent
    span, ascending, and coefficients C (m x r) with C^T GB C = I."""
    ga = _c(ga, np.float64); gb = _c(gb, np.float64); m = ga.shape[0]
    theta = np.empty(m); c = np.empty((m, m))
    r = lib().or_rayleigh_ritz(m, _ptr(ga), _ptr(gb), _ptr(theta), _ptr(c))
    return theta[:r].copy(), c.reshape(-1)[:m * r].reshape(m, r).copy()
