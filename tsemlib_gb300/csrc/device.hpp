// Device-resident objects behind the C handles.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "common.hpp"
#include "physics.hpp"
#include "space.hpp"

namespace tsem {

// Chebyshev smoothing interval [lmax / kChebRange, lmax] of D^-1 A on every p-multigrid
// level (matrix-free mixed solver and assembled FP64 Chebyshev p-MG alike).  Coarsening
// the degree by two leaves much of the middle of the spectrum to the smoother, so the
// interval reaches far below the usual lmax / 30: on the 3.05 M DOF p = 6 Poisson
// problem the mixed solver takes 47 inner iterations with 4 steps per level and
// lmax / 200, against 67 with 3 steps and lmax / 30 (56 with 4 steps and lmax / 30).
constexpr double kChebRange = 200.0;

struct DevCsr {
    int64_t n = 0, nnz = 0;
    DBuf<int64_t> rowptr;
    DBuf<int> col;
    DBuf<double> val;
    DBuf<double> diag;      // cached diagonal (refreshed after value changes)
    int spmv_variant = -1;  // SpMV launch shape chosen by the autotuner (-1: untuned)
    float spmv_ms = 0.0f;
    std::vector<float> spmv_shape_ms;  // the autotuner's time of every launch shape, ms per launch
    // the autotuner's check of every shape against the FP64 shape 0 on a random x:
    // max over rows of |y_shape - y_0| / (|A| |x|)_row
    std::vector<double> spmv_shape_err;
    // values and the SpMV input as FP32 (hi, lo) pairs for the FP32-pipe SpMV
    // shapes: rebuilt from val after every change of the values
    mutable DBuf<float2> vsplit, xsplit;
    mutable bool split_ok = false;
    void values_changed() { split_ok = false; }
    void refresh_diag(cudaStream_t s);
};

struct ReferenceMatrices {
    int n_loc = 0;
    std::vector<double> mass, stiff;          // host copies, dense [n][n] and [6][n][n]
    // assembly lists: structural (a, c) pairs with their values
    DBuf<int> mass_pairs, stiff_pairs;        // packed a * n_loc + c
    DBuf<double> mass_vals, stiff_vals;       // [np], [np][6]
    int64_t n_mass_pairs = 0, n_stiff_pairs = 0;
};

struct SpaceDevice {
    bool ready = false;
    DBuf<int> t_n, t_ind;
    DBuf<double> t_val;
    DBuf<double> xyz, volume;
    DBuf<int> ele_node;
    DBuf<double> x3, w3;                      // reference quadrature
};

}  // namespace tsem

struct tsem_space_s {
    tsem::SpaceHost host;
    tsem::Quadrature quad;
    tsem::SpaceDevice dev;
    tsem::PhysicsDevice phys;
    std::unique_ptr<tsem::ReferenceMatrices> ref;
    std::unique_ptr<tsem::PatternCandidates> cand;
    cudaStream_t stream = nullptr;
    int device = 0;
};

struct tsem_csr_s {
    tsem::DevCsr m;
    cudaStream_t stream = nullptr;
    int device = 0;
};

namespace tsem {
void ensure_stream(cudaStream_t* s, int* device);
void space_upload(tsem_space_s* sp);
void space_reference(tsem_space_s* sp);
void space_assemble(tsem_space_s* sp, int which, DevCsr& out);
void csr_spmv(const DevCsr& A, const double* x, double* y, cudaStream_t s);
// rows/columns g with map[g] >= 0 of `fine`, renumbered to map[g] (nc of them)
void principal_submatrix(const DevCsr& fine, const std::vector<int>& map, int64_t nc, DevCsr& C, cudaStream_t s);
// time every launch shape on A once and keep the fastest; with `reuse`, a matrix of a
// kind already tuned in this process (mean row length, size class) takes that shape
void spmv_autotune(DevCsr& A, cudaStream_t s, bool reuse = false);
// A.vsplit = A.val as FP32 (hi, lo) pairs, rebuilt when the values changed
void csr_split_values(const DevCsr& A, cudaStream_t s);
void csr_residual(const DevCsr& A, const double* x, double* r, const double* b, cudaStream_t s);
void physics_basis(tsem_space_s* sp);
void element_qpoints(tsem_space_s* sp, double* host_out);
void boundary_points(tsem_space_s* sp, int dim, double* out, int64_t* count);
void rhs(tsem_space_s* sp, const double* f_qp_host, double* rhs_host);
void rhs_device(tsem_space_s* sp, const double* f_qp, double* rhs, cudaStream_t s);
void neumann(tsem_space_s* sp, double* rhs_host, const double* g_host, int flag);
void dirichlet(tsem_space_s* sp, DevCsr& A, double* rhs_host, const double* uv, const double* ue, const double* uf,
               bool modify, int flag);
void zero_bc(tsem_space_s* sp, DevCsr* A, double* rhs_host, int flag);
void errors(tsem_space_s* sp, const double* sol_host, const double* uq_host, const double* guq_host, double* out);
// pattern of all element mode pairs (matrices with element-dependent dense blocks)
void space_pattern_full(tsem_space_s* sp, DevCsr& out);
// A (full-block pattern of sp) = sum_e |T_e| sum_q w_q V_e(q) phi_a(q) phi_c(q) through T_e
void assemble_potential(tsem_space_s* sp, const double* v_qp_host, DevCsr& A);
void assemble_potential_device(tsem_space_s* sp, const double* v_qp, DevCsr& A, cudaStream_t s);
// values of the FE function `sol` at the element quadrature points, [E][nq]
void eval_qp(tsem_space_s* sp, const double* sol_host, double* out_host);
void eval_qp_device(tsem_space_s* sp, const double* sol, double* out, cudaStream_t s);
void density(tsem_space_s* sp, const double* states_host, int k, const double* occ, double* out_host);
void density_device(tsem_space_s* sp, const double* states, int k, const double* occ, double* out, cudaStream_t s);
double density_l2_difference(tsem_space_s* sp, const double* u_host, const double* v_host, int k, const double* occ);
// calc_interpolation: modal interpolant from u at the boundary points of all vertices,
// edges and faces and at the element quadrature points
void interpolation(tsem_space_s* sp, const double* uv, const double* ue, const double* uf, const double* u_qp,
                   double* out_host);
// dst += alpha src; src's pattern must lie inside dst's
void csr_axpy(DevCsr& dst, double alpha, const DevCsr& src, cudaStream_t s);
}  // namespace tsem
