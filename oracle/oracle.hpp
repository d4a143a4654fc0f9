// TEST INFRASTRUCTURE ONLY -- CPU oracle for the TSEM discretise-and-solve path.
//
// This is a plain FP64 C++ restatement of TSEMLib's algorithms, used by tests/,
// by __graft_entry__.smoke() and by bench.py's CPU baseline leg as the checker.
// Nothing in the shipped library links, loads or calls it.  Each routine cites
// the TSEMLib source it restates (path:line within the TSEMLib project).
//
// Parity pins: the reference ships no golden outputs, and only its multi-index
// headers compile without AFEPack, deal.II and LAPACKE.  The oracle is pinned by
// (a) the output of those headers (include/Correspondence.h, Multiindex.h) built
// from the reference tree into oracle/_ref, stored as tests/golden/multiindex_M12.txt;
// (b) the reference's own data files: the face re-orientation table, the tabulated
// quadrature rules and the 1-D Gauss tables its collapsed rules are built from
// (tests/golden); (c) LAPACK's dsygvx, which the reference calls for its
// Rayleigh-Ritz step; (d) analytic reference-matrix entries cross-checked by exact
// quadrature; (e) the global<->local round trip the reference prints as a
// self-test; (f) analytic eigenvalues and manufactured solutions.  Assembled
// values, DOF order and iteration counts stay unpinned against reference outputs.
#pragma once
#include <cstdint>
#include <vector>
#include <array>
#include <string>

namespace tsem_oracle {

// ---------------------------------------------------------------- index algebra
// Lexicographic numbering of multi-indices alpha in N^3, |alpha| <= M, ordered by
// total degree, then by (alpha2+alpha3) ascending, then alpha3 ascending.
// Restates include/Correspondence.h:64-109.
struct MultiIndexTable {
    int M = 0;
    int n = 0;
    std::vector<std::array<int, 3>> num2idx;
    void init(int order);
    static int number(int a0, int a1, int a2);  // position of alpha, any M
    static int count_upto(int deg) { return (deg + 1) * (deg + 2) * (deg + 3) / 6; }
};

// binomial coefficient with the reference's convention (returns 1 when n < m),
// src/Miscellaneous.cpp:165-172
int binom_ref(int n, int m);

// --------------------------------------------------------- Jacobi coefficients
// src/Miscellaneous.cpp:175-468
double coef_a(int al, int be, int ind, int k);
double coef_b(int al, int be, int ind, int k);
double coef_c(int al, int be, int ind, int k);
double coef_d(int al, int be, int k);
double coef_e(int al, int be, int ind, int k);
double coef_g(int al, int be, int ind, int k);
double coef_D(int ind_derivative, int ind_variation, int l1, int l2, int l3);
double jacobi_gen(int al, int be, int k, double x);  // :510-542

// ------------------------------------------------------------------ quadrature
// Collapsed (Duffy) tensor Gauss rule with q points per direction on the unit
// simplices, weights normalised to unit measure.  Restates src/QuadInfo.cpp:63-119
// (1-D Gauss-Legendre nodes are computed here instead of read from a table).
struct Quadrature {
    int q = 0;
    std::vector<double> x1, w1;              // 1-D: barycentric [p][0], weight
    std::vector<std::array<double, 3>> b2;   // 2-D barycentric (x, y, 1-x-y)
    std::vector<double> w2;
    std::vector<std::array<double, 3>> x3;   // 3-D reference points
    std::vector<double> w3;
    void build(int q);
};
void gauss_legendre01(int q, std::vector<double>& x, std::vector<double>& w);

// ------------------------------------------------------------- local basis
// Local transform J_alpha -> phi (src/BuildSpace.cpp:296-377) and basis values.
struct LocalBasis {
    int M = 0, n_loc = 0;
    MultiIndexTable mi;
    std::vector<std::vector<int>> tl;      // transform_local
    std::vector<std::vector<double>> wtl;  // weight_transform_local
    void init(int M);
    // value of J_alpha (Jacobi products, src/BuildSpace.cpp:24-51) at a 3-D point
    void jacobi_values(const double* pt, double* out) const;
    // actual basis phi at a 3-D point (src/BuildSpace.cpp:418-424)
    void basis_values(const double* pt, double* out) const;
    // gradient of J_alpha (src/BuildSpace.cpp:189-290), out[n_loc][3]
    void jacobi_gradients(const double* pt, double* out) const;
    void basis_gradients(const double* pt, double* out) const;
};

// --------------------------------------------------------- reference matrices
// Sparse n_loc x n_loc matrices stored as (pattern, value) with the structural
// pattern of the reference (deal.II square patterns keep the diagonal).
struct RefSparse {
    int n = 0;
    std::vector<std::vector<int>> cols;     // sorted column lists (diag included)
    std::vector<std::vector<double>> vals;  // same shape
    void init(int n_) { n = n_; cols.assign(n, {}); vals.assign(n, {}); }
    void add_pattern(int r, int c);
    void finalize_pattern();                // sort/unique + add diagonal
    void add_value(int r, int c, double v); // value must be in pattern
    double get(int r, int c) const;
};
struct RefMatrices {
    int M = 0, n_loc = 0;
    RefSparse mass_jac;             // in the Jacobi basis (Discretize.cpp:121-340)
    RefSparse mass;                 // actual basis (:435-464)
    RefSparse stiff_jac[6];         // Discretize.cpp:848-1175
    RefSparse stiff[6];             // actual basis (:1224-1293)
    void build(const LocalBasis& lb);
};

// -------------------------------------------------------------- face table
// Re-expression of a face mode under the 6 vertex permutations of a face
// (the reference reads it from include/quad_info/Info_Interpolate_More,
// src/BuildSpace.cpp:1704-1771).  Loaded from a golden extract.
struct FaceTable {
    int M_tab = 0, nf_tab = 0;
    // [var][dof][edge 0..2] -> list of (edge dof index, value)
    std::vector<std::vector<std::array<std::vector<std::pair<int, double>>, 3>>> edge;
    // [var][dof] -> list of (face dof index, value)
    std::vector<std::vector<std::vector<std::pair<int, double>>>> face;
    bool load(const std::string& path);
};

// ------------------------------------------------------------------- mesh
// AFEPack-style topology: face k of a tet is opposite its vertex k, edge k of a
// face is opposite its vertex k.
struct Mesh {
    int nv = 0, ne = 0, nf = 0, nt = 0;
    std::vector<double> xyz;       // [nv][3]
    std::vector<int> edge_v;       // [ne][2]
    std::vector<int> face_v;       // [nf][3]
    std::vector<int> face_e;       // [nf][3]
    std::vector<int> tet_v;        // [nt][4]
    std::vector<int> tet_f;        // [nt][4]
    std::vector<int> mark_v, mark_e, mark_f;  // boundary marks
    std::vector<int> femdof_v, femdof_e;      // fem-dof number of vertices/edges
};

// ------------------------------------------------------------------ CSR
struct Csr {
    int n = 0;
    std::vector<int64_t> rowptr;
    std::vector<int> col;           // diagonal first in every row, then ascending
    std::vector<double> val;
    int64_t find(int r, int c) const;
    void vmult(const double* x, double* y) const;
};

// ------------------------------------------------------------ the space
struct Space {
    int M = 0, n_loc = 0;
    LocalBasis lb;
    RefMatrices ref;
    Quadrature quad;
    const Mesh* mesh = nullptr;
    int n_geo[4] = {0, 0, 0, 0};
    int n_dof_geo[4] = {0, 0, 0, 0};
    int n_geo_total = 0, n_dof = 0, n_ele = 0;
    // geometry info (src/BuildSpace.cpp:436-655)
    std::vector<int> ele_node, ele_edge, ele_face;   // [E][4], [E][6], [E][4]
    std::vector<int> type_edge;                       // [E][6] 0 same, 1 reversed
    std::vector<int> type_face, type_face_inv;        // [E][4]
    std::vector<int> edge_node;                       // number_node[0], [ne][2]
    std::vector<int> face_node, face_edge;            // number_node[1], number_edge
    std::vector<uint8_t> face_same;                   // flag_sameorder_edgeonface [nf][3]
    std::vector<double> volume;                       // |T|
    // global numbering (src/BuildSpace.cpp:872-948)
    std::vector<int> location_geometry, location_actualdof;
    // per-element transform global -> local, padded [E][n_loc][max_dep]
    int max_dep = 0;
    std::vector<int> t_n;          // [E][n_loc]
    std::vector<int> t_ind;        // [E][n_loc][max_dep]
    std::vector<double> t_val;     // [E][n_loc][max_dep]
    // boundary marks per geometry (flag_bm)
    std::vector<int> flag_bm[3];

    void build(const Mesh& m, int M, const FaceTable& ft, int quad_q);
    int geo_first_dof(int dim, int idx) const;
    void sum_dof(std::vector<int>& out) const;           // Miscellaneous.cpp:557-587
    void assemble_stiff(Csr& A) const;                    // Discretize.cpp:1297-1395
    void assemble_mass(Csr& A) const;                     // Discretize.cpp:522-593
    // local coefficients of a global vector on element e
    void gather(int e, const double* u, double* loc) const;
};

// -------------------------------------------------------------- solvers
struct PcgStats { int iterations = 0; double residual_l1 = 0, init_l1 = 0, residual_l2 = 0; int status = 0; };

struct PMG {
    int n_project = 0;
    std::vector<int> n_dof_layer;
    std::vector<std::vector<int>> core_at;     // [level][fine dof] -> coarse or -1
    std::vector<Csr> A;                        // A[0] = fine (copy), A[i] coarse
    void init(const Csr& fine, int p, const std::vector<int>& sum_dof, int order_step);
    void vcycle(double* x, const double* r, int smooth) const;  // TSEMSolver.cpp:1120-1183
};

void gs_forward(const Csr& A, double* x, const double* r, int steps);
void gs_backward(const Csr& A, double* x, const double* r, int steps);
void gs_symmetric(const Csr& A, double* x, const double* r, int steps);

// flag: 0 none, 1 Jacobi, 4 p-MG.  rel_tol > 0 switches to the relative
// 2-norm stopping rule; otherwise the reference's absolute l1 rule is used.
PcgStats solve_pcg(const Csr& A, double* x, const double* b, double tol_abs_l1,
                   double rel_tol, int max_step, int flag, const PMG* pmg, int smooth, double omega = 1.0);

}  // namespace tsem_oracle
