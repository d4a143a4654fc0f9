/*
 * tsem_gpu.h -- C ABI of the GB300 TSEM discretise-and-solve library (libtsemgpu.so).
 *
 * Drop-in for the hot path of TSEMLib: the TSEM<double> space and discretisation
 * (include/TetrahedralSEM.h:29-331) and the TSEMSolver<double> solvers
 * (include/TSEMSolver.h:57-98).  Each entry point names the reference function it
 * replaces.  Plain pointers and sizes only; every call returns a tsem_status and
 * never prints.  Host pointers are copied; the library owns its device memory.
 * Calls on distinct handles may run concurrently from different host threads.
 *
 * Mesh input replaces AFEPack's RegularMesh<3> + P2 FEMSpace<double,3>: the
 * same relations the reference reads from them (face k of a tetrahedron is
 * opposite its vertex k, edge k of a face is opposite its vertex k; the P2
 * DOF numbers of vertices and edges fix the global DOF order,
 * src/BuildSpace.cpp:906-948).
 */
#ifndef TSEM_GPU_H
#define TSEM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tsem_status {
    TSEM_OK = 0,
    TSEM_MAXIT = 1,        /* iteration limit reached (reference prints "failed to converge", TSEMSolver.cpp:1925) */
    TSEM_BREAKDOWN = 2,    /* p^T A p <= 0 or a singular projected problem */
    TSEM_NONFINITE = 3,    /* NaN/Inf met in the iteration */
    TSEM_OOM_REFUSED = 4,  /* device allocation refused or over the memory budget */
    TSEM_TIMEOUT = 5,      /* a bounded device wait gave up */
    TSEM_INVALID = 6,      /* inconsistent input */
    TSEM_CUDA_ERROR = 7,   /* CUDA runtime error */
    TSEM_NO_DEVICE = 8     /* no usable CUDA device */
} tsem_status;

typedef struct tsem_space_s* tsem_space;
typedef struct tsem_csr_s* tsem_csr;
typedef struct tsem_solver_s* tsem_solver;

typedef struct tsem_mesh {
    int32_t nv, ne, nf, nt;
    const double* xyz;       /* [nv][3] vertex coordinates (mesh.point(i)) */
    const int32_t* edge_v;   /* [ne][2] */
    const int32_t* face_v;   /* [nf][3] */
    const int32_t* face_e;   /* [nf][3] edge opposite face vertex k (geometry(2,f).boundary(k)) */
    const int32_t* tet_v;    /* [nt][4] */
    const int32_t* tet_f;    /* [nt][4] face opposite vertex k (geometry(3,t).boundary(k)) */
    const int32_t* mark_v;   /* [nv] boundary marks (boundaryMark()), may be NULL */
    const int32_t* mark_e;   /* [ne] may be NULL */
    const int32_t* mark_f;   /* [nf] may be NULL */
    const int32_t* femdof_v; /* [nv] P2 DOF number of every vertex */
    const int32_t* femdof_e; /* [ne] P2 DOF number of every edge; together a permutation of 0..nv+ne-1 */
} tsem_mesh;

/* Message of the last failing call on this thread. */
const char* tsem_last_error(void);
/* number of kernels the library has launched in this process so far (a
 * diagnostic counter, no counterpart in TSEMLib) */
int64_t tsem_kernel_launches(void);

/* ---------------------------------------------------------------- space
 * TSEM<double>::init(p, q, mesh, fem_space) without the matrices
 * (TSEM::init_lazy, src/Initialize.cpp:84-97): numbering, geometry info and the
 * global->local transforms; collapsed Gauss rule with quad_q points per direction
 * (build_quad_info, src/QuadInfo.cpp:63-119).  Host work only. */
tsem_status tsem_space_create(const tsem_mesh* mesh, int32_t p, int32_t quad_q, tsem_space* out);
/* read_quad_info (src/QuadInfo.cpp:13-60): replace the space's quadrature by a
 * tabulated rule, as TSEM<double>::init does with its default tables (20 / 130 / 923
 * points, include/TetrahedralSEM.h:144-147): 1-D points x1 [n1] in [0, 1] (the first
 * barycentric coordinate), 2-D barycentric points b2 [n2][3], 3-D reference points
 * x3 [n3][3], weights w1 / w2 / w3 normalised to unit measure.  Everything that
 * integrates with the space's rule (right-hand sides, boundary data, errors,
 * interpolation, the potential matrix) uses it from then on; the reference-element
 * matrices are exact and do not depend on it. */
tsem_status tsem_space_set_quadrature(tsem_space s, int32_t n1, const double* x1, const double* w1, int32_t n2,
                                      const double* b2, const double* w2, int32_t n3, const double* x3,
                                      const double* w3);
/* ends a space (the lifetime of a TSEM<double> object) */
void tsem_space_destroy(tsem_space s);
/* info[15]: n_dof, n_loc, n_ele, max_dep, nq3, nq2, nq1, n_geo[4], n_dof_geo[4] -- the sizes
 * TSEM<double> holds (n_dof_total, n_index, n_element, n_q_point, n_geometry,
 * n_dof_geometry; include/TetrahedralSEM.h:34-65) */
tsem_status tsem_space_info(tsem_space s, int64_t* info);
/* location_geometry / location_actualdof (src/BuildSpace.cpp:939-948), [nv+ne+nf+nt] each */
tsem_status tsem_space_numbering(tsem_space s, int32_t* location_geometry, int32_t* location_actualdof);
/* transform_{n,ind,val}_global2local (TetrahedralSEM.h:124-126) padded: [E][n_loc], [E][n_loc][max_dep] */
tsem_status tsem_space_transform(tsem_space s, int32_t* t_n, int32_t* t_ind, double* t_val);
/* type_projection for edges [E][6] and faces [E][4], type_projection_inv [E][4],
 * number_node edges [ne][2] / faces [nf][3], number_edge [nf][3],
 * flag_sameorder_edgeonface [nf][3], element volume [E] (src/BuildSpace.cpp:436-646) */
tsem_status tsem_space_geometry(tsem_space s, int8_t* type_edge, int8_t* type_face, int8_t* type_face_inv,
                                int32_t* edge_node, int32_t* face_node, int32_t* face_edge, uint8_t* face_same,
                                double* volume);
/* calc_sum_dof (src/Miscellaneous.cpp:557-587) */
tsem_status tsem_space_sum_dof(tsem_space s, int32_t* sum_dof);
/* quadrature rule (QPoint, QPoint_Barycentric, Weight; include/TetrahedralSEM.h:42-44):
 * x3 [nq3][3], w3 [nq3], b2 [nq2][3], w2 [nq2], x1 [nq1], w1 [nq1]; any may be NULL */
tsem_status tsem_space_quadrature(tsem_space s, double* x3, double* w3, double* b2, double* w2, double* x1, double* w1);
/* physical 3-D quadrature points of every element, [E][nq3][3] (GPU): the points
 * calc_rhs and the error routines evaluate their functions at (src/Discretize.cpp:1397-1418,
 * src/CalcError.cpp:64-92) */
tsem_status tsem_element_qpoints(tsem_space s, double* out);
/* boundary evaluation points of every vertex / edge / face, in the layout the
 * Dirichlet and Neumann entry points expect; *count = number of points */
tsem_status tsem_boundary_points(tsem_space s, int32_t dim, double* out, int64_t* count);
/* boundary marks of every vertex / edge / face (dim 0, 1, 2), the geometries of
 * tsem_boundary_points in the same order; *count = number of geometries.  The
 * Dirichlet and Neumann entry points read the values of the geometries their flag
 * selects, so a caller may evaluate its boundary function at those points only. */
tsem_status tsem_geometry_marks(tsem_space s, int32_t dim, int32_t* out, int64_t* count);

/* The multi-index numbering of order M (Correspondence<3>::number2index and
 * index2number, include/Correspondence.h:64-109): for each number i below
 * (M+1)(M+2)(M+3)/6, alpha[3 i .. 3 i + 2] = the multi-index of number i (ordered by
 * total degree, then alpha1 + alpha2, then alpha2) and number[i] = the number of that
 * multi-index back again.  Either array may be NULL.  0 <= M <= 40. */
tsem_status tsem_multiindex(int32_t M, int32_t* alpha, int32_t* number);

/* Face re-orientation table derived for order p (the coefficients the reference
 * reads from Info_Interpolate_More, src/BuildSpace.cpp:1704-1771).  With NULL
 * arrays returns *n_entries; entries are (var, local dof, kind 0 edge / 1 face,
 * edge k, index, value). */
tsem_status tsem_face_table(int32_t p, int64_t* n_entries, int32_t* var, int32_t* dof, int32_t* kind, int32_t* edge_k,
                            int32_t* index, double* value);

/* ---------------------------------------------------------- discretisation
 * Reference-element matrices in the actual basis, dense [n_loc][n_loc]:
 * which 0 = mass (build_mass_matrix_init, src/Discretize.cpp:121-464), 1..6 = the
 * six stiffness matrices (build_stiff_matrix_init, :845-1294).  Computed on the
 * GPU by exact quadrature; entries outside the reference's structural pattern are 0. */
tsem_status tsem_reference_matrix(tsem_space s, int32_t which, double* dense, uint8_t* pattern);
/* build_stiff_matrix (which 0, src/Discretize.cpp:1297-1395) / build_mass_matrix
 * (which 1, :522-665): GPU assembly into a device CSR, diagonal first in each row. */
tsem_status tsem_assemble(tsem_space s, int32_t which, tsem_csr* out);
/* The device CSR that stands in for deal.II's SparseMatrix<double> / SparsityPattern
 * (TSEM<double>::stiff_matrix, mass_matrix, include/TetrahedralSEM.h:217-218; rows
 * diagonal first, then ascending columns, as SparsityPattern::compress leaves them):
 * size and nonzeros, export to and import from host arrays, copy
 * (SparseMatrix::copy_from), destroy. */
tsem_status tsem_csr_info(tsem_csr A, int64_t* n, int64_t* nnz);
tsem_status tsem_csr_export(tsem_csr A, int64_t* rowptr, int32_t* col, double* val);
tsem_status tsem_csr_import(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, tsem_csr* out);
tsem_status tsem_csr_copy(tsem_csr A, tsem_csr* out);
void tsem_csr_destroy(tsem_csr A);
/* y = A x (SparseMatrix::vmult); device != 0 means x, y are device pointers used on
 * `stream` (a cudaStream_t, NULL = the library stream) */
tsem_status tsem_csr_spmv(tsem_csr A, const double* x, double* y, int32_t device, void* stream);
/* The SpMV autotuner's record for A (no reference counterpart: the launch shape is a
 * property of this library).  shape = the chosen launch shape (-1 before the first
 * tsem_csr_spmv), ms = its time per launch; shape_ms and shape_err (either may be
 * NULL) receive up to cap per-shape times and per-shape deviations from the FP64
 * shape 0 on the tuner's random x (max over rows of |y - y_0| / (|A| |x|)_row; the
 * tuner refuses a matrix on which any shape exceeds 1e-13), *count the number of
 * shapes timed. */
tsem_status tsem_csr_spmv_tuning(tsem_csr A, int32_t* shape, float* ms, float* shape_ms, double* shape_err,
                                 int32_t cap, int32_t* count);

/* calc_rhs(rhs, value_f) (src/Discretize.cpp:1397-1418): f at the element
 * quadrature points [E][nq3]; rhs [n_dof] is overwritten. */
tsem_status tsem_rhs(tsem_space s, const double* f_qp, double* rhs);
/* Neumann load (impose_boundary_condition(rhs, mesh, g, flag), :2011-2063): g at
 * the 2-D boundary points of every face; adds to rhs. */
tsem_status tsem_neumann(tsem_space s, double* rhs, const double* g_face_pts, int32_t flag);
/* Dirichlet data by modal projection plus symmetric elimination
 * (impose_boundary_condition(A, rhs, value_bnd, modify, flag), :1683-1776).
 * u at the boundary points of vertices / edges / faces.  The closure of every
 * flagged face must be flagged (the reference's projection reads edge values).
 * modify = 0 leaves A unchanged and gives rhs as modify = 1 would: boundary rows
 * diag * value, other rows minus their boundary columns times the values.  On a matrix
 * whose boundary couplings are already zero that is the reference's result; on one
 * that still has them the reference's sequential loop (:1752-1773) leaves an
 * order-dependent rhs instead, a case no reference driver uses. */
tsem_status tsem_dirichlet(tsem_space s, tsem_csr A, double* rhs, const double* u_v, const double* u_e,
                           const double* u_f, int32_t modify, int32_t flag);
/* impose_zero_boundary_condition (:1466-1499 matrix, :1533-1545 rhs); A or rhs may be NULL */
tsem_status tsem_zero_bc(tsem_space s, tsem_csr A, double* rhs, int32_t flag);
/* calc_l2_error / calc_l2_error_gradient (src/CalcError.cpp:64-92, :126-189):
 * u [E][nq3], grad u [E][nq3][3] at the element quadrature points; out[0] = L2,
 * out[1] = L2 norm of the gradient error. */
tsem_status tsem_errors(tsem_space s, const double* sol, const double* u_qp, const double* gu_qp, double* out);

/* ------------------------------------------------------------------ solvers */
/* build_mass_V_matrix (src/Discretize.cpp:668-756): M_V = sum_e |T_e| sum_q w_q
 * V_e(q) phi_a(q) phi_c(q) through T_e, V given at the element quadrature points
 * ([E][nq], the order of tsem_element_qpoints).  The pattern holds every element
 * mode pair (a superset of the stiffness and mass patterns).  *inout == NULL
 * creates the matrix; a matrix this call made for the same space is refilled in
 * place (same pattern, new values). */
tsem_status tsem_assemble_potential(tsem_space s, const double* v_qp, tsem_csr* inout);
/* calc_interpolation (src/Interpolation.cpp:104-216): modal interpolant of u given at
 * the points of tsem_boundary_points for dimensions 0, 1, 2 (all vertices, edges and
 * faces) and at the element quadrature points (tsem_element_qpoints); out [n_dof] */
tsem_status tsem_interpolation(tsem_space s, const double* u_v, const double* u_e, const double* u_f,
                               const double* u_qp, double* out);
/* values of the FE function `sol` (n_dof coefficients) at the element quadrature
 * points, out [E][nq] (the per-element evaluation of calc_val_qp_onElement,
 * src/PointInfo.cpp:2013-2022) */
tsem_status tsem_eval_qp(tsem_space s, const double* sol, double* out);
/* tsem_eval_qp, tsem_rhs and tsem_assemble_potential on device arrays (the FE
 * coefficients, the [E][nq] point values, the rhs), enqueued on `stream` (NULL =
 * the space's stream) where the inputs are ready; no host copy of the [E][nq]
 * arrays.  tsem_assemble_potential_device returns when the matrix is complete. */
tsem_status tsem_eval_qp_device(tsem_space s, const double* sol, double* out, void* stream);
/* calc_density (src/PointInfo.cpp:72-91): rho = sum_j occ[j] psi_j^2 at the element
 * quadrature points, out [E][nq3]; the k states (1 <= k <= 64) one after another,
 * states [k][n_dof] (host arrays; _device: device arrays, occ on the host). */
tsem_status tsem_density(tsem_space s, const double* states, int32_t k, const double* occ, double* out);
tsem_status tsem_density_device(tsem_space s, const double* states, int32_t k, const double* occ, double* out,
                                void* stream);
/* calc_density_l2_difference (src/CalcError.cpp:703-735): the L2 norm of
 * sum_j occ[j] (u_j^2 - v_j^2); u, v [k][n_dof] host arrays. */
tsem_status tsem_density_l2_difference(tsem_space s, const double* u, const double* v, int32_t k, const double* occ,
                                       double* out);
tsem_status tsem_rhs_device(tsem_space s, const double* f_qp, double* rhs, void* stream);
tsem_status tsem_assemble_potential_device(tsem_space s, const double* v_qp, tsem_csr* inout, void* stream);
/* dst += alpha src (deal.II SparseMatrix::add(factor, matrix)); src's pattern must
 * lie inside dst's (TSEM_INVALID otherwise) */
tsem_status tsem_csr_add(tsem_csr dst, double alpha, tsem_csr src);

typedef struct tsem_solver_opts {
    int32_t precond;        /* 0 none, 1 Jacobi (default of solve_PCG), 2 SOR, 3 SSOR, 4 p-multigrid */
    int32_t pmg_order_step; /* orders dropped per level: 1 = p, p-1, ..., 1 (TSEMSolver.cpp:44-55) */
    int32_t smooth_steps;   /* GS sweeps per level (the `var` argument of solve_PCG) */
    int32_t smoother;       /* 0 exact lexicographic Gauss-Seidel (reference), 1 Chebyshev-Jacobi */
    double tol_abs_l1;      /* reference stopping rule: ||r||_1 < tol */
    double tol_rel;         /* > 0: stop when ||r||_2 <= tol_rel ||b||_2 instead */
    int32_t max_iter;       /* PCG iterations (outer refinement steps for the mixed solver) */
    double inner_tol;       /* mixed solver: residual reduction of an FP32 inner solve (0 = 1e-6); the last
                               refinement step asks only for what the target still needs */
    double omega;           /* SOR / SSOR relaxation in (0, 2) for precond 2, 3 (0 = 1); their sweep count
                               is smooth_steps (the ite_step of solve_PCG) */
} tsem_solver_opts;

typedef struct tsem_stats {
    int32_t iterations;
    int32_t status;         /* tsem_status of the solve */
    double residual_l1;     /* ||r||_1 at exit */
    double init_l1;
    double residual_rel;    /* ||r||_2 / ||b||_2 at exit */
    double device_ms;       /* time spent on the device stream */
} tsem_stats;

/* TSEMSolver<double>::init_PMG (src/TSEMSolver.cpp:36-135) when precond == 4:
 * p-multigrid levels {sum_dof <= q}, injection transfers, principal-submatrix
 * coarse operators.  A must outlive the solver. */
tsem_status tsem_solver_create(tsem_csr A, const int32_t* sum_dof, int32_t p, const tsem_solver_opts* opts,
                               tsem_solver* out);
void tsem_solver_destroy(tsem_solver sv);
/* solve_PCG (src/TSEMSolver.cpp:1776-1929); b, x host arrays, x holds the initial guess */
tsem_status tsem_solve_pcg(tsem_solver sv, const double* b, double* x, tsem_stats* st);
/* same on device arrays, enqueued on `stream` (NULL = library stream); returns when done */
tsem_status tsem_solve_pcg_device(tsem_solver sv, const double* b, double* x, tsem_stats* st, void* stream);
/* solve_PMG (src/TSEMSolver.cpp:1446-1536): V-cycles on x (host, in/out) until
 * ||A x - b||_1 < tol or max_step cycles; st->iterations counts the cycles.  The
 * coarsest level takes ite_PMG's (smooth+1)/2 symmetric sweeps. */
tsem_status tsem_solve_pmg(tsem_solver sv, const double* b, double* x, double tol, int32_t max_step, tsem_stats* st);
/* one ite_PMG V-cycle (src/TSEMSolver.cpp:1120-1183) on host arrays: x in/out, r */
tsem_status tsem_pmg_vcycle(tsem_solver sv, double* x, const double* r);

/* Block LOBPCG for the k smallest eigenpairs of A x = lambda M x, A the solver's
 * operator and M a CSR matrix of the same size (TSEMSolver::solve_LOBPCG,
 * src/TSEMSolver.cpp:2225-2406 for a block, :2071-2222 for k = 1).  X: host,
 * column-major n x k (column j at X + j n): the initial block in, the
 * M-orthonormal Ritz vectors out; lambda: k values out, ascending.  The residual
 * block is preconditioned with the solver's p-multigrid V-cycle (FP64 for a plain
 * solver, the FP32 matrix-free V-cycle for a mixed one; Jacobi without p-MG).
 * The block products, Gram matrices and Ritz combinations are FP64 on (hi, lo)
 * FP32 pairs (about 2^-48 per product, compensated sums); the Rayleigh-Ritz
 * problem is FP64 (scaling, pivoted Cholesky, triangular solves) with its Jacobi
 * rotations on pairs.  Stops when the first n_want pairs reach
 * ||A x - lambda M x|| <= tol |lambda| ||M x|| (st.residual_rel: the largest of
 * those ratios) or after max_it iterations (TSEM_MAXIT); st.init_l1 holds the most
 * Jacobi sweeps any Rayleigh-Ritz step took. */
tsem_status tsem_solve_lobpcg(tsem_solver sv, tsem_csr M, int32_t k, int32_t n_want, double* X, double* lambda,
                              double tol, int32_t max_it, tsem_stats* st);
/* same for the pencil (A, M) with an operator A other than the solver's (same size),
 * the solver supplying only the preconditioner: a Kohn-Sham Hamiltonian 1/2 K + M_V
 * preconditioned by the p-multigrid V-cycle of K (SCFIteration.cpp:297, 391) */
tsem_status tsem_solve_lobpcg_pencil(tsem_solver precond, tsem_csr A, tsem_csr M, int32_t k, int32_t n_want, double* X,
                                     double* lambda, double tol, int32_t max_it, tsem_stats* st);
/* same with X on the device, enqueued on `stream` (NULL = solver stream); returns when done */
tsem_status tsem_solve_lobpcg_device(tsem_solver sv, tsem_csr M, int32_t k, int32_t n_want, double* X,
                                     double* lambda, double tol, int32_t max_it, tsem_stats* st, void* stream);

/* Mixed-precision matrix-free solver for the stiffness system of `s` with the
 * Dirichlet DOFs of boundary mark `dirichlet_flag` eliminated (as A_bc after
 * tsem_dirichlet / tsem_zero_bc).  No reference counterpart: it replaces the
 * reference's PCG loop on A_bc (src/TSEMSolver.cpp:1776-1929) by FP64 iterative
 * refinement around an FP32 PCG whose operator and p-multigrid are applied per
 * element; A_bc (FP64 CSR) gives the outer residual.  Solve with
 * tsem_solve_pcg / tsem_solve_pcg_device; stats.iterations counts inner PCG
 * iterations and stats.init_l1 the outer refinement steps. */
tsem_status tsem_solver_create_mixed(tsem_space s, tsem_csr A_bc, int32_t dirichlet_flag, const tsem_solver_opts* opts,
                                     tsem_solver* out);
/* y = A_level x with the matrix-free operator of a mixed solver (level 0 = order
 * p); host arrays of the level size.  low_precision != 0 selects the BF16
 * tensor-core GEMM where the level has one (the smoother's operator). */
tsem_status tsem_mf_apply(tsem_solver sv, int32_t level, int32_t low_precision, const double* x, double* y,
                          int64_t* level_n);
/* same on FP32 device arrays, enqueued on `stream` (NULL = solver stream); no synchronisation */
tsem_status tsem_mf_apply_device(tsem_solver sv, int32_t level, int32_t low_precision, const float* x, float* y,
                                 void* stream);
/* z = one V-cycle of the mixed solver's matrix-free p-multigrid applied to r, from
 * z = 0 (the preconditioner of its inner PCG; ite_PMG, src/TSEMSolver.cpp:1120-1183,
 * with the Chebyshev-Jacobi smoother), for ncol FP32 columns of the fine-level size
 * n stored n apart (device arrays).  The block runs as one V-cycle whose launches
 * cover all columns; each column's result equals that of a one-column call.
 * Enqueued on `stream` (NULL = solver stream). */
tsem_status tsem_mf_vcycle_device(tsem_solver sv, int32_t ncol, const float* r, float* z, void* stream);
/* Kernel-level timing of one matrix-free apply on `level` (no reference
 * counterpart): CUDA-event device time of its gather, element-GEMM and scatter
 * kernels averaged over `reps` applies to a fixed vector, and their algorithmic
 * work.  out[9] = {ms gather, ms GEMM, ms scatter, bytes gather, bytes GEMM,
 * flops GEMM, bytes scatter, ms and bytes of the scatter with a Chebyshev step of
 * the smoother fused in (the p-multigrid's most frequent launch)}. */
tsem_status tsem_mf_profile(tsem_solver sv, int32_t level, int32_t low_precision, int32_t reps, double* out);
/* y = A_level x, the same operator as tsem_mf_apply_device with low_precision = 0,
 * for callers that may not allocate device memory during the call (a host whose
 * memory is all in its own pool, a serving loop that must not stall on an
 * allocator).  The arithmetic differs: FP32 CUDA-core element GEMMs on every level
 * and an atomic scatter, so the result agrees with tsem_mf_apply_device to FP32
 * rounding (about 1e-6 relative) and may differ from run to run in the last bits.
 * The element scratch is one static device array of TSEM_NOALLOC_SCRATCH_BYTES; a
 * level whose scratch, 4 * (64 + 2 * ceil64(ceil64(E) * n_local_modes)) bytes with
 * E the element count rounded up to an odd multiple of 32, is larger is rejected
 * with TSEM_INVALID (the message gives the bytes the level needs).  x and y must
 * not overlap (TSEM_INVALID): y is cleared before x is read.  The solver's device
 * must be current.  The first call on a device looks up the array's address; make
 * it before any stream capture.  All calls on a device share the array: calls that
 * overlap in time race and must be ordered (one stream, or events).  A bounded wait
 * that gives up inside the call leaves y all NaN.  TSEMLib has no counterpart of
 * this call. */
#define TSEM_NOALLOC_SCRATCH_BYTES (16u << 20)
tsem_status tsem_mf_apply_device_noalloc(tsem_solver sv, int32_t level, const float* x, float* y, void* stream);

/* ------------------------------------------------------------ batched solves
 * Several mixed solvers' systems solved together (no TSEMLib counterpart; the
 * reference solves one system per solve_PCG call, src/TSEMSolver.cpp:1776-1929).
 * Each system keeps its own FP64 refinement; the inner PCG iterations of all systems
 * run in lockstep rounds, and solvers of the same order whose levels have the same
 * shape share every V-cycle launch: the BF16 tensor-core element GEMM runs over a
 * ragged table of all their element tiles, the scatters and vector updates over all
 * their DOFs.  A system's result equals what tsem_solve_pcg gives it to the solve
 * tolerance (the inner products sum in another order).  b[i], x[i]: the systems'
 * right-hand sides and initial guesses (solutions on return), host arrays when
 * device == 0, device arrays on the solvers' device otherwise; every solver once, all
 * on the current device; st (may be NULL) receives n statistics.  Returns TSEM_OK or
 * the first system's failing status. */
tsem_status tsem_solve_batch(const tsem_solver* sv, int32_t n, const double* const* b, double* const* x, int32_t device,
                             void* stream, tsem_stats* st);

/* Continuous batching (the request loop's submit / poll / cancel; no TSEMLib
 * counterpart).  A batch runs the systems submitted to it as tsem_solve_batch does,
 * and new systems join at the next round while others are in flight:
 * tsem_batch_submit (any thread) queues the system of a mixed solver, b and x device
 * arrays on the batch's device, x the initial guess, and returns a ticket;
 * tsem_batch_poll (polls from several threads take turns) admits the queued
 * systems, runs one round (one inner iteration of every system in its inner solve,
 * the refinement steps that are due) and reports up to cap retired systems (ticket,
 * statistics; cancelled ones with TSEM_INVALID) and the number still in flight;
 * tsem_batch_cancel retires a system at the next poll.  A solver may have one system
 * in a batch at a time and must outlive it; b and x must stay valid until its ticket
 * is reported. */
typedef struct tsem_batch_s* tsem_batch;
tsem_status tsem_batch_create(void* stream, tsem_batch* out);
void tsem_batch_destroy(tsem_batch bt);
tsem_status tsem_batch_submit(tsem_batch bt, tsem_solver sv, const double* b, double* x, int64_t* ticket);
tsem_status tsem_batch_poll(tsem_batch bt, int32_t cap, int64_t* tickets, tsem_stats* stats, int32_t* n_done,
                            int32_t* n_in_flight);
tsem_status tsem_batch_cancel(tsem_batch bt, int64_t ticket);

/* Test hook (no TSEMLib counterpart): the number of polls after which a bounded
 * device wait of the matrix-free kernels gives up, on the current device; polls <= 0
 * restores the default 2^26.  A wait that gives up records where it did, the kernel
 * waits (with the full limit) for its own copies and MMAs in flight, frees its
 * tensor memory and returns; the call then fails with TSEM_TIMEOUT and the context
 * stays usable.  With a limit of a few polls the next matrix-free solve gives up on
 * its first waits, which is how the failure path is tested without a GPU fault. */
tsem_status tsem_debug_wait_limit(int64_t polls);

/* Test hook of the checked build (the library compiled with -DTSEM_CHECK; no TSEMLib
 * counterpart).  There the matrix-free operator's gathers and scatters and the mixed
 * solver's FP32 SpMVs check every index they read from a table against the length
 * of the vector it addresses; an index outside records the first failure (a code
 * naming the kernel, and the index) and its access is skipped -- nothing traps -- and
 * the solve then fails with TSEM_INVALID.  shrink >= 1 divides every bound (a value
 * above 1 makes valid indices fail, to exercise that path with every remaining
 * access inside its vector); code / index receive the first failure since the last
 * call, which is cleared; checked = 1 in the checked build, 0 otherwise (where the
 * checks compile to nothing and code stays 0). */
tsem_status tsem_debug_bounds(int32_t shrink, int32_t* code, int64_t* index, int32_t* checked);

/* ------------------------------------------------------------------ service
 * Request loop (no TSEMLib counterpart; the reference solves one problem per
 * process).  tsem_serve replays a stream of requests at their arrival times:
 * `workers` threads take them in arrival order as soon as the device-memory
 * budget admits their estimated footprint, each request on its own CUDA streams,
 * so their work overlaps on the device; each request's mesh, operators, multigrid
 * hierarchy and Krylov state stay resident until it retires.  A request is the
 * unit cube, N^3 Kuhn-split sub-cubes with seeded node jitter, order p, zero
 * Dirichlet conditions on every face; Poisson requests have a seeded sum of eight
 * Gaussians as right-hand side, eigen requests ask for the n_eig smallest pairs of
 * the Laplacian (mass matrix as B, guard vectors added).  plain = 0 solves with
 * the mixed matrix-free solver, 1 with the plain FP64 CSR solver. */
typedef struct tsem_request {
    int64_t id;
    int32_t kind;          /* 0 Poisson, 1 Laplace eigenpairs */
    int32_t n_cube;        /* N */
    int32_t order;         /* p >= 2 */
    int32_t n_eig;         /* eigen: wanted pairs */
    double jitter;         /* node jitter, fraction of the sub-cube width */
    uint64_t seed;
    double tol;            /* Poisson: relative residual */
    double tol_eig;        /* eigen: relative residual of the wanted pairs (0 = 1e-8) */
    double arrival_s;      /* arrival time, seconds from the start of the stream */
    double* x_out;         /* optional host array receiving the Poisson solution */
} tsem_request;

typedef struct tsem_result {
    int64_t id;
    int32_t status;        /* tsem_status of the request */
    int32_t iterations;
    int64_t n_dof;
    double queued_s;       /* start - arrival */
    double latency_s;      /* completion - arrival */
    double finish_s;       /* completion, from the start of the stream */
    double setup_s;        /* mesh, space, assembly, boundary conditions, solver set-up */
    double solve_s;
    double residual;       /* relative residual reached */
    double checksum;       /* sum of the solution (first eigenvector) entries */
    double norm2;          /* sum of their squares */
    double lambda0, lambda_last;   /* eigen: smallest and n_eig-th eigenvalue */
} tsem_result;

typedef struct tsem_serve_opts {
    int32_t workers;              /* requests in flight at most */
    int32_t plain;                /* 1: plain FP64 CSR solver */
    int32_t realtime;             /* 1: honour arrival times; 0: all arrive at time 0 */
    double memory_budget_bytes;   /* admission budget (0 = 150 GB) */
} tsem_serve_opts;

tsem_status tsem_serve(const tsem_request* reqs, int64_t n_req, const tsem_serve_opts* opts, tsem_result* results);

#ifdef __cplusplus
}
#endif

#endif /* TSEM_GPU_H */
