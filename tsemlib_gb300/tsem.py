"""Python mirror of TSEMLib's TSEM<double> / TSEMSolver<double> interface on the GPU.

Names and argument meanings follow include/TetrahedralSEM.h and
include/TSEMSolver.h; callbacks of the reference (``double f(double*)``) become
vectorised Python callables evaluated at the points the library reports.  All
numerical work runs in libtsemgpu.so on the GPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import TsemError, c_array, check, ptr, stream_ptr  # noqa: F401  (TsemError re-exported)
from .mesh import TetMesh


class SparseMatrix:
    """Device CSR matrix, diagonal first in every row (deal.II convention)."""

    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.tsem_csr_destroy(self.h)
            self.h = None

    @classmethod
    def from_arrays(cls, rowptr, col, val):
        rowptr = c_array(rowptr, np.int64); col = c_array(col, np.int32); val = c_array(val, np.float64)
        h = ctypes.c_void_p()
        check(_lib.lib().tsem_csr_import(len(rowptr) - 1, ptr(rowptr), ptr(col), ptr(val), ctypes.byref(h)))
        return cls(h)

    def add(self, factor, matrix: "SparseMatrix"):
        """self += factor * matrix (deal.II SparseMatrix::add); matrix's pattern must lie
        inside this one's."""
        check(_lib.lib().tsem_csr_add(self.h, float(factor), matrix.h))
        return self

    def copy(self):
        h = ctypes.c_void_p()
        check(_lib.lib().tsem_csr_copy(self.h, ctypes.byref(h)))
        return SparseMatrix(h)

    def shape(self):
        n = ctypes.c_int64(); nnz = ctypes.c_int64()
        check(_lib.lib().tsem_csr_info(self.h, ctypes.byref(n), ctypes.byref(nnz)))
        return n.value, nnz.value

    @property
    def n(self):
        return self.shape()[0]

    @property
    def nnz(self):
        return self.shape()[1]

    def arrays(self):
        n, nnz = self.shape()
        rp = np.empty(n + 1, np.int64); c = np.empty(nnz, np.int32); v = np.empty(nnz, np.float64)
        check(_lib.lib().tsem_csr_export(self.h, ptr(rp), ptr(c), ptr(v)))
        return rp, c, v

    def vmult(self, x):
        """y = A x (SparseMatrix::vmult)."""
        x = c_array(x, np.float64)
        y = np.empty_like(x)
        check(_lib.lib().tsem_csr_spmv(self.h, ptr(x), ptr(y), 0, None))
        return y

    def vmult_device(self, x_ptr, y_ptr, stream=None):
        check(_lib.lib().tsem_csr_spmv(self.h, ptr(x_ptr), ptr(y_ptr), 1, stream_ptr(stream)))

    def spmv_tuning(self, with_errors=False):
        """The SpMV autotuner's record: (chosen launch shape, its ms per launch, ms per
        launch of every shape timed); shape -1 before the first vmult.  with_errors adds
        every shape's largest deviation from the FP64 shape, per row relative to
        (|A| |x|)_row, on the tuner's random x."""
        shape, count = ctypes.c_int32(0), ctypes.c_int32(0)
        ms = ctypes.c_float(0.0)
        buf = np.zeros(64, np.float32)
        err = np.zeros(64, np.float64)
        check(_lib.lib().tsem_csr_spmv_tuning(self.h, ctypes.byref(shape), ctypes.byref(ms), ptr(buf), ptr(err),
                                              len(buf), ctypes.byref(count)))
        k = min(count.value, len(buf))
        if with_errors:
            return shape.value, ms.value, buf[:k].tolist(), err[:k].tolist()
        return shape.value, ms.value, buf[:k].tolist()


def read_quad_tables(n_quadrature_point, quad_filename):
    """The three quadrature tables of read_quad_info (src/QuadInfo.cpp:13-60), parsed as
    the reference parses them: n_quadrature_point[d] records of "x w" (1-D, x in
    [-1, 1] mapped to the barycentric (x + 1) / 2), "x y w" (2-D, barycentric x, y;
    the third coordinate 1 - x - y) and "x y z w" (3-D reference points).  Returns the
    arrays of TSEM.set_quadrature."""
    out = {}
    for d, (n, fn) in enumerate(zip(n_quadrature_point, quad_filename)):
        with open(fn) as f:
            tok = np.array(f.read().split()[: int(n) * (d + 2)], dtype=np.float64).reshape(int(n), d + 2)
        pts, w = tok[:, : d + 1], tok[:, d + 1].copy()
        if d == 0:
            out["x1"], out["w1"] = (pts[:, 0] + 1.0) / 2.0, w
        elif d == 1:
            out["b2"], out["w2"] = np.column_stack([pts[:, 0], pts[:, 1], 1.0 - pts[:, 0] - pts[:, 1]]), w
        else:
            out["x3"], out["w3"] = pts.copy(), w
    return out


class TSEM:
    """TSEM<double>(M, q, mesh, fem_space): space, stiffness and mass matrices.

    ``lazy=True`` mirrors ``init_lazy`` (no matrices)."""

    def __init__(self, polynomial_order: int, qinfo_order: int, mesh: TetMesh, lazy: bool = False):
        L = _lib.lib()
        self.mesh = mesh
        self.M = polynomial_order
        m = mesh
        self._keep = [c_array(m.xyz, np.float64), c_array(m.edge_v, np.int32), c_array(m.face_v, np.int32),
                      c_array(m.face_e, np.int32), c_array(m.tet_v, np.int32), c_array(m.tet_f, np.int32),
                      c_array(m.mark_v, np.int32), c_array(m.mark_e, np.int32), c_array(m.mark_f, np.int32),
                      c_array(m.femdof_v, np.int32), c_array(m.femdof_e, np.int32)]
        k = self._keep
        desc = _lib.Mesh(m.nv, m.ne, m.nf, m.nt, *[ptr(a) for a in k])
        h = ctypes.c_void_p()
        check(L.tsem_space_create(ctypes.byref(desc), polynomial_order, qinfo_order, ctypes.byref(h)))
        self.h = h
        info = np.zeros(15, np.int64)
        check(L.tsem_space_info(self.h, ptr(info)))
        self.n_dof_total, self.n_index, self.n_element, self.max_dep = (int(x) for x in info[:4])
        self.n_q_point = [int(info[6]), int(info[5]), int(info[4])]     # 1-D, 2-D, 3-D as in the reference
        self.n_geometry = [int(x) for x in info[7:11]]
        self.n_dof_geometry = [int(x) for x in info[11:15]]
        self.stiff_matrix = None
        self.mass_matrix = None
        if not lazy:
            self.build_stiff_matrix()
            self.build_mass_matrix()

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.tsem_space_destroy(self.h)
            self.h = None

    # ---------------------------------------------------------------- structure
    def numbering(self):
        ng = sum(self.n_geometry)
        lg = np.empty(ng, np.int32); la = np.empty(ng, np.int32)
        check(_lib.lib().tsem_space_numbering(self.h, ptr(lg), ptr(la)))
        return lg, la

    def transform(self):
        E, nl, md = self.n_element, self.n_index, self.max_dep
        tn = np.empty((E, nl), np.int32); ti = np.empty((E, nl, md), np.int32); tv = np.empty((E, nl, md))
        check(_lib.lib().tsem_space_transform(self.h, ptr(tn), ptr(ti), ptr(tv)))
        return tn, ti, tv

    def geometry(self):
        m, E = self.mesh, self.n_element
        out = dict(type_edge=np.empty(6 * E, np.int8), type_face=np.empty(4 * E, np.int8),
                   type_face_inv=np.empty(4 * E, np.int8), edge_node=np.empty(2 * m.ne, np.int32),
                   face_node=np.empty(3 * m.nf, np.int32), face_edge=np.empty(3 * m.nf, np.int32),
                   face_same=np.empty(3 * m.nf, np.uint8), volume=np.empty(E))
        check(_lib.lib().tsem_space_geometry(self.h, *[ptr(v) for v in out.values()]))
        return out

    def write_coef(self, src, filename):
        """write_coef (src/Miscellaneous.cpp:108-127): "M<TAB>n_dof" then every value
        of every vector, one per line, 14 significant digits."""
        vecs = [np.asarray(src)] if np.ndim(src) == 1 else [np.asarray(v) for v in src]
        with open(filename, "w") as f:
            f.write(f"{self.M}\t{self.n_dof_total}\n")
            for v in vecs:
                f.write("".join(f"{x:.14g}\n" for x in v))

    def read_coef(self, filename, n_vectors=1):
        """read_coef (src/Miscellaneous.cpp:35-105): coefficients of order M' onto this
        space, geometry by geometry (the first modes of every vertex, edge, face and
        interior block; order lifting when M' < M).  Geometry blocks of order M' hold
        binom(M'-1, d) modes; the reference's binomial returns 1 when M'-1 < d
        (src/Miscellaneous.cpp:165-172), here it is 0.  Returns one vector, or an
        [n_vectors, n_dof] array."""
        from math import comb
        with open(filename) as f:
            tok = f.read().split()
        Mi, ni = int(tok[0]), int(tok[1])
        data = np.array(tok[2:2 + ni * n_vectors], dtype=np.float64).reshape(n_vectors, ni)
        cnt_i = [comb(Mi - 1, d) if Mi - 1 >= d else 0 for d in range(4)]
        cnt = [comb(self.M - 1, d) if self.M - 1 >= d else 0 for d in range(4)]
        lg, la = self.numbering()
        ng = self.n_geometry
        dims = np.concatenate([np.full(ng[d], d) for d in range(4)])
        dim_sorted = np.empty_like(dims)
        dim_sorted[lg] = dims
        start_i = np.concatenate([[0], np.cumsum(np.array(cnt_i)[dim_sorted])[:-1]])
        out = np.zeros((n_vectors, self.n_dof_total))
        for d in range(4):
            locs = np.arange(sum(ng[:d]), sum(ng[:d + 1]))
            srt = lg[locs]
            for j in range(min(cnt_i[d], cnt[d])):
                out[:, la[srt] + j] = data[:, start_i[srt] + j]
        return out[0] if n_vectors == 1 else out

    def calc_sum_dof(self):
        out = np.empty(self.n_dof_total, np.int32)
        check(_lib.lib().tsem_space_sum_dof(self.h, ptr(out)))
        return out

    def quadrature(self):
        n1, n2, n3 = self.n_q_point
        x3 = np.empty((n3, 3)); w3 = np.empty(n3); b2 = np.empty((n2, 3)); w2 = np.empty(n2)
        x1 = np.empty(n1); w1 = np.empty(n1)
        check(_lib.lib().tsem_space_quadrature(self.h, *[ptr(a) for a in (x3, w3, b2, w2, x1, w1)]))
        return dict(x3=x3, w3=w3, b2=b2, w2=w2, x1=x1, w1=w1)

    def read_quad_info(self, n_quadrature_point, quad_filename):
        """read_quad_info (src/QuadInfo.cpp:13-60): replace the collapsed Gauss rule by
        the tabulated rules of three files, read as the reference reads them
        (read_quad_tables); the reference's defaults are the 20 / 130 / 923-point
        tables of include/TetrahedralSEM.h:144-147."""
        rule = read_quad_tables(n_quadrature_point, quad_filename)
        self.set_quadrature(**rule)

    def set_quadrature(self, x1, w1, b2, w2, x3, w3):
        """Install a tabulated rule (tsem_space_set_quadrature): x1 [n1] in [0, 1],
        b2 [n2, 3] barycentric, x3 [n3, 3], weights of unit total."""
        a = [c_array(v, np.float64) for v in (x1, w1, b2, w2, x3, w3)]
        check(_lib.lib().tsem_space_set_quadrature(self.h, len(a[1]), ptr(a[0]), ptr(a[1]), len(a[3]), ptr(a[2]),
                                                   ptr(a[3]), len(a[5]), ptr(a[4]), ptr(a[5])))
        self._rule = a
        self.n_q_point = [len(a[1]), len(a[3]), len(a[5])]

    def element_qpoints(self):
        out = np.empty((self.n_element, self.n_q_point[2], 3))
        check(_lib.lib().tsem_element_qpoints(self.h, ptr(out)))
        return out

    def boundary_points(self, dim):
        """Evaluation points of every vertex / edge / face (dim 0, 1, 2), [count, 3]."""
        cache = self.__dict__.setdefault("_bpoints", {})
        if dim not in cache:
            cnt = ctypes.c_int64()
            check(_lib.lib().tsem_boundary_points(self.h, dim, None, ctypes.byref(cnt)))
            out = np.empty((cnt.value, 3))
            check(_lib.lib().tsem_boundary_points(self.h, dim, ptr(out), ctypes.byref(cnt)))
            out.flags.writeable = False
            cache[dim] = out
        return cache[dim].copy()

    def geometry_marks(self, dim):
        """Boundary marks of every vertex / edge / face (dim 0, 1, 2)."""
        cache = self.__dict__.setdefault("_gmarks", {})
        if dim not in cache:
            cnt = ctypes.c_int64()
            check(_lib.lib().tsem_geometry_marks(self.h, dim, None, ctypes.byref(cnt)))
            out = np.empty(cnt.value, np.int32)
            check(_lib.lib().tsem_geometry_marks(self.h, dim, ptr(out), ctypes.byref(cnt)))
            cache[dim] = out
        return cache[dim]

    def _boundary_values(self, u, dim, flag, exact=False):
        """u at the boundary points of dimension dim whose geometry the flag selects
        (-1: any boundary mark, otherwise that mark; exact: that mark only), zero at
        the others (the Dirichlet and Neumann kernels do not read them)."""
        self.boundary_points(dim)
        pts = self._bpoints[dim]
        marks = self.geometry_marks(dim)
        on = (marks != 0) if (flag == -1 and not exact) else (marks == flag)
        out = np.zeros(len(pts))
        if len(marks) and on.any():
            sel = np.repeat(on, len(pts) // len(marks))
            out[sel] = np.asarray(u(pts[sel]), dtype=np.float64).reshape(-1)
        return out

    def reference_matrix(self, which: int):
        n = self.n_index
        d = np.empty((n, n)); pat = np.empty((n, n), np.uint8)
        check(_lib.lib().tsem_reference_matrix(self.h, which, ptr(d), ptr(pat)))
        return d, pat.astype(bool)

    # ----------------------------------------------------------- discretisation
    def _assemble(self, which):
        h = ctypes.c_void_p()
        check(_lib.lib().tsem_assemble(self.h, which, ctypes.byref(h)))
        return SparseMatrix(h)

    def build_stiff_matrix(self):
        self.stiff_matrix = self._assemble(0)
        return self.stiff_matrix

    def build_mass_matrix(self):
        self.mass_matrix = self._assemble(1)
        return self.mass_matrix

    def calc_rhs(self, f=None, value_f=None):
        """calc_rhs(rhs, fem_space, f) or calc_rhs(rhs, value_f)."""
        if value_f is None:
            value_f = f(self.element_qpoints())
        value_f = c_array(value_f, np.float64)
        out = np.empty(self.n_dof_total)
        check(_lib.lib().tsem_rhs(self.h, ptr(value_f), ptr(out)))
        return out

    def impose_neumann(self, rhs, g, flag_boundary: int = 2):
        """impose_boundary_condition(rhs, mesh, g, flag) -- Neumann load, in place."""
        gv = self._boundary_values(g, 2, flag_boundary, exact=True)
        check(_lib.lib().tsem_neumann(self.h, ptr(rhs), ptr(gv), flag_boundary))
        return rhs

    def impose_boundary_condition(self, A: SparseMatrix, rhs, u, flag_modify_matrix=True, flag_boundary=1):
        """impose_boundary_condition(A, rhs, mesh, u, modify, flag) -- Dirichlet, in place.
        With flag_modify_matrix false A is left as it is and rhs becomes the right-hand
        side that true gives (the reference's false branch agrees on a matrix whose
        boundary couplings are already zero)."""
        if flag_boundary == -2:
            vb = [c_array(u(self.boundary_points(d)), np.float64) for d in range(3)]
        else:
            vb = [self._boundary_values(u, d, flag_boundary) for d in range(3)]
        check(_lib.lib().tsem_dirichlet(self.h, A.h, ptr(rhs), ptr(vb[0]), ptr(vb[1]), ptr(vb[2]),
                                        int(flag_modify_matrix), flag_boundary))
        return rhs

    def build_mass_V_matrix(self, value_V=None, func=None, out: SparseMatrix | None = None):
        """build_mass_V_matrix (src/Discretize.cpp:668-843): (V phi_i, phi_j) with V given
        at the element quadrature points ([E][nq]) or as a function of points.  `out`
        (a matrix this method returned for the space) is refilled in place."""
        if value_V is None:
            value_V = func(self.element_qpoints())
        v = c_array(value_V, np.float64)
        h = ctypes.c_void_p(out.h.value if out is not None else None)
        check(_lib.lib().tsem_assemble_potential(self.h, ptr(v), ctypes.byref(h)))
        return out if out is not None else SparseMatrix(h)

    def calc_interpolation(self, func):
        """calc_interpolation (src/Interpolation.cpp:104-216): the modal interpolant of func
        (vertex values, edge / face / interior modal projections)."""
        pts = [c_array(func(self.boundary_points(d)), np.float64) for d in range(3)]
        uq = c_array(func(self.element_qpoints()), np.float64)
        out = np.empty(self.n_dof_total)
        check(_lib.lib().tsem_interpolation(self.h, ptr(pts[0]), ptr(pts[1]), ptr(pts[2]), ptr(uq), ptr(out)))
        return out

    def value_qp(self, sol):
        """Values of the FE function `sol` at the element quadrature points, [E, nq]."""
        sol = c_array(sol, np.float64)
        out = np.empty((self.n_element, self.n_q_point[2]))
        check(_lib.lib().tsem_eval_qp(self.h, ptr(sol), ptr(out)))
        return out

    def calc_density(self, psi, n_occupation):
        """calc_density (src/PointInfo.cpp:72-91): sum_j occ_j psi_j^2 at the element
        quadrature points, [E, nq].  psi: k vectors (a list, or a k x n_dof array)."""
        st = c_array(np.atleast_2d(np.asarray(psi, dtype=np.float64)), np.float64)
        occ = c_array(n_occupation, np.float64)
        assert st.shape == (len(occ), self.n_dof_total)
        out = np.empty((self.n_element, self.n_q_point[2]))
        check(_lib.lib().tsem_density(self.h, ptr(st), len(occ), ptr(occ), ptr(out)))
        return out

    def calc_density_l2_difference(self, u, v, n_occupation):
        """calc_density_l2_difference (src/CalcError.cpp:703-735): || sum_j occ_j (u_j^2 -
        v_j^2) ||_L2; u, v: k vectors each."""
        uu = c_array(np.atleast_2d(np.asarray(u, dtype=np.float64)), np.float64)
        vv = c_array(np.atleast_2d(np.asarray(v, dtype=np.float64)), np.float64)
        occ = c_array(n_occupation, np.float64)
        assert uu.shape == vv.shape == (len(occ), self.n_dof_total)
        out = ctypes.c_double()
        check(_lib.lib().tsem_density_l2_difference(self.h, ptr(uu), ptr(vv), len(occ), ptr(occ), ctypes.byref(out)))
        return out.value

    # ---- device-array forms (pointers to FP64 device memory; stream None = the space's)
    def value_qp_device(self, sol_ptr, out_ptr, stream=None):
        """value_qp on device arrays: sol [n_dof] -> out [E, nq]."""
        check(_lib.lib().tsem_eval_qp_device(self.h, ptr(sol_ptr), ptr(out_ptr), stream_ptr(stream)))

    def calc_density_device(self, psi_ptr, n_occupation, out_ptr, stream=None):
        """calc_density on device arrays: psi [k][n_dof] -> out [E, nq]; occupations on the host."""
        occ = c_array(n_occupation, np.float64)
        check(_lib.lib().tsem_density_device(self.h, ptr(psi_ptr), len(occ), ptr(occ), ptr(out_ptr),
                                             stream_ptr(stream)))

    def calc_rhs_device(self, f_ptr, out_ptr, stream=None):
        """calc_rhs(rhs, value_f) on device arrays: f [E, nq] -> rhs [n_dof]."""
        check(_lib.lib().tsem_rhs_device(self.h, ptr(f_ptr), ptr(out_ptr), stream_ptr(stream)))

    def build_mass_V_matrix_device(self, v_ptr, out: SparseMatrix | None = None, stream=None):
        """build_mass_V_matrix with V [E, nq] in device memory; `out` is refilled in place."""
        h = ctypes.c_void_p(out.h.value if out is not None else None)
        check(_lib.lib().tsem_assemble_potential_device(self.h, ptr(v_ptr), ctypes.byref(h), stream_ptr(stream)))
        return out if out is not None else SparseMatrix(h)

    def impose_zero_boundary_condition(self, A: SparseMatrix | None = None, rhs=None, flag_boundary=1):
        check(_lib.lib().tsem_zero_bc(self.h, None if A is None else A.h, ptr(rhs), flag_boundary))

    def calc_errors(self, sol, u, grad_u):
        """(calc_l2_error, calc_l2_error_gradient) against exact u and grad u."""
        q = self.element_qpoints()
        uq = c_array(u(q), np.float64); gq = c_array(grad_u(q), np.float64)
        sol = c_array(sol, np.float64)
        out = np.empty(2)
        check(_lib.lib().tsem_errors(self.h, ptr(sol), ptr(uq), ptr(gq), ptr(out)))
        return float(out[0]), float(out[1])


def kernel_launches() -> int:
    """Kernels the library has launched in this process so far."""
    return int(_lib.lib().tsem_kernel_launches())


def face_table(p: int):
    """The derived face re-orientation table as flat arrays."""
    L = _lib.lib()
    n = ctypes.c_int64()
    check(L.tsem_face_table(p, ctypes.byref(n), None, None, None, None, None, None))
    arr = [np.empty(n.value, np.int32) for _ in range(5)] + [np.empty(n.value)]
    check(L.tsem_face_table(p, ctypes.byref(n), *[ptr(a) for a in arr]))
    return dict(var=arr[0], dof=arr[1], kind=arr[2], edge_k=arr[3], index=arr[4], value=arr[5])


def multiindex(M: int):
    """Correspondence<3> of order M (include/Correspondence.h:64-109): the
    multi-index of every number, [n][3], and each multi-index's number back."""
    n = (M + 1) * (M + 2) * (M + 3) // 6
    alpha = np.empty((n, 3), np.int32)
    number = np.empty(n, np.int32)
    check(_lib.lib().tsem_multiindex(M, ptr(alpha), ptr(number)))
    return alpha, number


class TSEMSolver:
    """TSEMSolver<double>: PCG with none / Jacobi / p-multigrid preconditioning."""

    SMOOTHERS = {"gs": 0, "chebyshev": 1}

    def __init__(self):
        self._pmg = None
        self._solvers = {}

    def init_PMG(self, sp_matrix: SparseMatrix, polynomial_order: int, sum_dof, order_step: int = 1,
                 smoother: str = "gs"):
        """init_PMG(A, mass, p, sum_dof); the mass argument of the reference is unused there."""
        self._pmg = dict(A=sp_matrix, p=polynomial_order, sum_dof=c_array(sum_dof, np.int32), step=order_step,
                         smoother=self.SMOOTHERS[smoother])
        self._solvers.clear()

    def _solver(self, A, precond, smooth, tol, tol_rel, max_step, omega=0.0):
        key = (id(A), precond, smooth, tol, tol_rel, max_step, omega)
        sv = self._solvers.get(key)
        if sv is None:
            pm = self._pmg or {}
            opts = _lib.SolverOpts(precond, pm.get("step", 1), smooth, pm.get("smoother", 0), tol, tol_rel, max_step, 0.0,
                                   omega)
            h = ctypes.c_void_p()
            sd = pm.get("sum_dof") if precond == 4 else None
            check(_lib.lib().tsem_solver_create(A.h, ptr(sd), pm.get("p", 1), ctypes.byref(opts), ctypes.byref(h)))
            sv = _Handle(h)
            self._solvers[key] = sv
        return sv

    def solve_PCG(self, sp_matrix: SparseMatrix, x, r, tol=1e-8, max_step=100000, flag_preconditioner=1,
                  ite_step=1, var=1, tol_rel=0.0):
        """solve_PCG(A, x, r, tol, max_step, flag, ite_step, var): x updated in place; returns stats.
        flag 2 (SOR) / 3 (SSOR): var is omega and ite_step the sweeps; flag 4: var is the
        smoothing steps of the V-cycle."""
        if flag_preconditioner == 4 and self._pmg is None:
            raise ValueError("init_PMG must precede flag_preconditioner == 4")
        sor = flag_preconditioner in (2, 3)
        smooth = int(var) if flag_preconditioner == 4 else (int(ite_step) if sor else 1)
        sv = self._solver(sp_matrix, flag_preconditioner, smooth, tol, tol_rel, max_step, float(var) if sor else 0.0)
        r = c_array(r, np.float64)
        st = _lib.Stats()
        rc = _lib.lib().tsem_solve_pcg(sv.h, ptr(r), ptr(x), ctypes.byref(st))
        check(rc, allow=(1, 2, 3))
        return st.as_dict()

    def solve_PCG_device(self, sp_matrix, x_ptr, r_ptr, tol=1e-8, max_step=100000, flag_preconditioner=1, var=1,
                         tol_rel=0.0, stream=None):
        smooth = int(var) if flag_preconditioner == 4 else 1
        sv = self._solver(sp_matrix, flag_preconditioner, smooth, tol, tol_rel, max_step)
        st = _lib.Stats()
        rc = _lib.lib().tsem_solve_pcg_device(sv.h, ptr(r_ptr), ptr(x_ptr), ctypes.byref(st),
                                              stream_ptr(stream))
        check(rc, allow=(1, 2, 3))
        return st.as_dict()

    def solve_LOBPCG(self, tsem, x, A: SparseMatrix, B: SparseMatrix, Flag_Output_Intermediate=False, tol=1e-8,
                     max_step=1000, n_want=None, smooth_step=2):
        """solve_LOBPCG(tsem, x, A, B, flag, tol, max_step) (src/TSEMSolver.cpp:2225-2406):
        block LOBPCG for the smallest pairs of A x = lambda B x.  x is an n x k array
        (columns = block vectors) or a list of k vectors, updated in place with the
        B-orthonormal Ritz vectors; returns (eigenvalues, stats).  The residual block is
        preconditioned with the p-multigrid V-cycle of init_PMG on A (Jacobi without
        it); the stop test is ||A x - lambda B x|| <= tol |lambda| ||B x|| for the first
        n_want (default all) pairs.  Flag_Output_Intermediate is accepted for the
        reference's signature; nothing is printed."""
        X, back = _block_in(x)
        n, k = X.shape
        precond = 4 if (self._pmg is not None and self._pmg["A"] is A) else 1
        sv = self._solver(A, precond, int(smooth_step) if precond == 4 else 1, 0.0, 0.0, 1)
        lam = np.empty(k)
        Xc = np.ascontiguousarray(X.T)          # column j of the block contiguous
        st = _lib.Stats()
        rc = _lib.lib().tsem_solve_lobpcg(sv.h, B.h, k, int(n_want or k), ptr(Xc), ptr(lam), float(tol),
                                          int(max_step), ctypes.byref(st))
        check(rc, allow=(1, 2))
        back(Xc.T)
        return lam, _lobpcg_stats(st)

    def solve_PMG(self, x, r, tol=1e-8, max_step=100000, smooth_step=2):
        """solve_PMG (src/TSEMSolver.cpp:1446-1536): stationary V-cycles on x (in place)
        until ||A x - r||_1 < tol; returns stats (iterations = cycles)."""
        pm = self._pmg
        if pm is None:
            raise ValueError("init_PMG must precede solve_PMG")
        sv = self._solver(pm["A"], 4, int(smooth_step), 0.0, 0.0, 1)
        r = c_array(r, np.float64)
        st = _lib.Stats()
        check(_lib.lib().tsem_solve_pmg(sv.h, ptr(r), ptr(x), float(tol), int(max_step), ctypes.byref(st)), allow=(1, 3))
        return st.as_dict()

    def solve_InversePower(self, x, A: SparseMatrix, B: SparseMatrix, Flag_Output_Intermediate=False, tol=1e-8,
                           max_step=1000, flag_preconditioner=1, var=1):
        """solve_InversePower (src/TSEMSolver.cpp:2042-2068): x <- A^-1 B x normalised in
        the B-norm, until the Rayleigh quotient x^T A x changes by less than tol; each
        solve is solve_PCG(A, x, B x, tol 1e-2, 100 max_step).  x (host) is updated in
        place; returns the eigenvalue estimate."""
        rhs = B.vmult(x)
        e_last = None
        e_now = 0.0
        for it in range(int(max_step)):
            self.solve_PCG(A, x, rhs, tol=tol * 1e-2, max_step=int(max_step) * 100,
                           flag_preconditioner=flag_preconditioner, var=var)
            rhs = B.vmult(x)
            c = float(rhs @ x)
            x /= np.sqrt(c)
            rhs /= np.sqrt(c)
            e_now = float(A.vmult(x) @ x)
            if it > 0 and abs(e_now - e_last) < tol:
                break
            e_last = e_now
        return e_now

    def ite_PMG(self, x, r, smooth_step=2):
        """One p-multigrid V-cycle (ite_PMG with ite_step = 1)."""
        pm = self._pmg
        sv = self._solver(pm["A"], 4, int(smooth_step), 0.0, 0.0, 1)
        x = c_array(x, np.float64).copy(); r = c_array(r, np.float64)
        check(_lib.lib().tsem_pmg_vcycle(sv.h, ptr(x), ptr(r)))
        return x


def _lobpcg_stats(st):
    """LOBPCG statistics: init_l1 carries the most Jacobi sweeps of any Rayleigh-Ritz step."""
    d = st.as_dict()
    d["jacobi_sweeps"] = int(st.init_l1)
    return d


def _block_in(x):
    """An n x k float64 view of a block given as an array or a list of vectors, and
    a function writing a result block back into it."""
    if isinstance(x, np.ndarray) and x.ndim == 2:
        X = np.asarray(x, dtype=np.float64)

        def back(Y):
            x[...] = Y
        return X, back
    cols = [np.asarray(v, dtype=np.float64) for v in x]
    X = np.stack(cols, axis=1)

    def back(Y):
        for j, v in enumerate(x):
            v[...] = Y[:, j]
    return X, back


class MixedSolver:
    """Matrix-free mixed-precision solver of A_bc x = b (no reference counterpart):
    FP64 iterative refinement around an FP32 PCG with a matrix-free p-multigrid."""

    def __init__(self, space: TSEM, A_bc: SparseMatrix, dirichlet_flag: int = 1, order_step: int = 2, smooth: int = 4,
                 tol_rel: float = 1e-10, inner_tol: float = 1e-6, max_outer: int = 40, tensor_smoother: bool = True):
        """tensor_smoother: the Chebyshev smoother applies the operator with the BF16
        tcgen05 GEMM (levels with >= 20 modes); the Krylov operator stays FP32."""
        opts = _lib.SolverOpts(4, order_step, smooth, 2 if tensor_smoother else 1, 0.0, tol_rel, max_outer, inner_tol)
        h = ctypes.c_void_p()
        check(_lib.lib().tsem_solver_create_mixed(space.h, A_bc.h, dirichlet_flag, ctypes.byref(opts), ctypes.byref(h)))
        self._h = _Handle(h)
        self.space = space
        self.A = A_bc

    def solve(self, x, b):
        """x (initial guess, updated in place), b host arrays; returns stats."""
        b = c_array(b, np.float64)
        st = _lib.Stats()
        rc = _lib.lib().tsem_solve_pcg(self._h.h, ptr(b), ptr(x), ctypes.byref(st))
        check(rc, allow=(1, 2, 3))
        d = st.as_dict()
        d["outer"] = int(st.init_l1)
        return d

    def solve_device(self, x_ptr, b_ptr, stream=None):
        st = _lib.Stats()
        rc = _lib.lib().tsem_solve_pcg_device(self._h.h, ptr(b_ptr), ptr(x_ptr), ctypes.byref(st),
                                              stream_ptr(stream))
        check(rc, allow=(1, 2, 3))
        d = st.as_dict()
        d["outer"] = int(st.init_l1)
        return d

    def level_size(self, level):
        n = ctypes.c_int64()
        check(_lib.lib().tsem_mf_apply(self._h.h, level, 0, None, None, ctypes.byref(n)))
        return n.value

    @property
    def num_levels(self):
        """Levels of the p-multigrid hierarchy (level 0 = order p, the last = order 1)."""
        n = ctypes.c_int64()
        L = 0
        while _lib.lib().tsem_mf_apply(self._h.h, L, 0, None, None, ctypes.byref(n)) == 0:
            L += 1
        return L

    def solve_LOBPCG(self, x, B: SparseMatrix, tol=1e-8, max_step=1000, n_want=None, A: SparseMatrix | None = None):
        """Block LOBPCG for A_bc x = lambda B x (or A x = lambda B x with another operator
        A of the same size) preconditioned by this solver's FP32 matrix-free p-multigrid
        V-cycle; Gram matrices and Rayleigh-Ritz in FP64.  x: n x k array or list of k
        vectors, updated in place; returns (eigenvalues, stats)."""
        X, back = _block_in(x)
        n, k = X.shape
        lam = np.empty(k)
        Xc = np.ascontiguousarray(X.T)
        st = _lib.Stats()
        if A is None:
            rc = _lib.lib().tsem_solve_lobpcg(self._h.h, B.h, k, int(n_want or k), ptr(Xc), ptr(lam), float(tol),
                                              int(max_step), ctypes.byref(st))
        else:
            rc = _lib.lib().tsem_solve_lobpcg_pencil(self._h.h, A.h, B.h, k, int(n_want or k), ptr(Xc), ptr(lam),
                                                     float(tol), int(max_step), ctypes.byref(st))
        check(rc, allow=(1, 2))
        back(Xc.T)
        return lam, _lobpcg_stats(st)

    def solve_LOBPCG_device(self, x_ptr, k, B: SparseMatrix, tol=1e-8, max_step=1000, n_want=None, stream=None):
        """Same on a device block (column-major n x k, FP64); returns (eigenvalues, stats)."""
        lam = np.empty(k)
        st = _lib.Stats()
        rc = _lib.lib().tsem_solve_lobpcg_device(self._h.h, B.h, int(k), int(n_want or k), ptr(x_ptr), ptr(lam),
                                                 float(tol), int(max_step), ctypes.byref(st), stream_ptr(stream))
        check(rc, allow=(1, 2))
        return lam, _lobpcg_stats(st)

    def profile(self, level=0, low_precision=True, reps=20):
        """CUDA-event times of the gather, element GEMM and scatter kernels of one apply
        on `level`, with their algorithmic bytes / flops, and the scatter with a
        Chebyshev step fused in (tsem_mf_profile)."""
        out = np.zeros(9)
        check(_lib.lib().tsem_mf_profile(self._h.h, level, int(low_precision), reps, ptr(out)))
        keys = ("ms_gather", "ms_gemm", "ms_scatter", "bytes_gather", "bytes_gemm", "flops_gemm", "bytes_scatter",
                "ms_scatter_cheb", "bytes_scatter_cheb")
        return dict(zip(keys, (float(v) for v in out)))

    def vcycle_device(self, ncol, r_ptr, z_ptr, stream=None):
        """z = V-cycle(r) of the matrix-free p-multigrid for ncol FP32 columns of the
        fine-level size stored one after another (device pointers)."""
        check(_lib.lib().tsem_mf_vcycle_device(self._h.h, int(ncol), ptr(r_ptr), ptr(z_ptr), stream_ptr(stream)))

    def apply_device(self, level, x_ptr, y_ptr, stream=None, low_precision=False):
        check(_lib.lib().tsem_mf_apply_device(self._h.h, level, int(low_precision), ptr(x_ptr), ptr(y_ptr),
                                              stream_ptr(stream)))

    def apply(self, level, x, low_precision=False):
        n = self.level_size(level)
        x = c_array(x, np.float64)
        assert x.shape == (n,)
        y = np.empty(n)
        check(_lib.lib().tsem_mf_apply(self._h.h, level, int(low_precision), ptr(x), ptr(y), None))
        return y


def solve_batch(solvers, bs, xs):
    """Solve the systems of several MixedSolvers together (tsem_solve_batch): the
    inner PCG iterations run in lockstep, solvers of the same order share every
    V-cycle launch through a ragged table of their elements and DOFs.  bs, xs: host
    arrays (xs: initial guesses, updated in place).  Returns one stats dict per system."""
    n = len(solvers)
    assert len(bs) == n and len(xs) == n and n >= 1
    b_arr = [c_array(b, np.float64) for b in bs]
    for sv, b, x in zip(solvers, b_arr, xs):
        assert isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous
        assert b.shape == x.shape
    hs = (ctypes.c_void_p * n)(*[sv._h.h.value for sv in solvers])
    bp = (ctypes.c_void_p * n)(*[b.ctypes.data for b in b_arr])
    xp = (ctypes.c_void_p * n)(*[x.ctypes.data for x in xs])
    st = (_lib.Stats * n)()
    rc = _lib.lib().tsem_solve_batch(hs, n, bp, xp, 0, None, st)
    check(rc, allow=(1, 2, 3))
    out = []
    for i in range(n):
        d = st[i].as_dict()
        d["outer"] = int(st[i].init_l1)
        out.append(d)
    return out


class _Handle:
    def __init__(self, h):
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.tsem_solver_destroy(self.h)
            self.h = None
