// TEST INFRASTRUCTURE ONLY -- CPU oracle (see oracle.hpp).
#pragma once
#include "oracle.hpp"

namespace tsem_oracle {

// 1-D/2-D bases used by the boundary projections (src/BuildSpace.cpp:53-170)
struct FaceBases {
    int nq1 = 0, nq2 = 0, ndE = 0, ndF = 0;
    std::vector<double> interp1;   // [nq1][ndE]   J^{1,1}_{l-2}
    std::vector<double> face_val;  // [nq2][ndF]   face modes on the 2-D reference triangle
    std::vector<double> interp2;   // [nq2][ndF]
    std::vector<double> add0, add1;  // [nq2][ndE]
    void build(const Space& S);
};

void element_qpoints(const Space& S, int e, std::vector<double>& out);
void boundary_points(const Space& S, int dim, std::vector<double>& out);
void calc_rhs(const Space& S, const double* f_qp, double* rhs);
void assemble_potential(const Space& S, const double* v_qp, Csr& out);
void impose_zero_bc(const Space& S, Csr* A, double* rhs, int flag);
void impose_dirichlet(const Space& S, const FaceBases& FB, Csr& A, double* rhs, const double* vb0,
                      const double* vb1, const double* vb2, bool modify, int flag);
void impose_neumann(const Space& S, const FaceBases& FB, double* rhs, const double* g2, int flag);
void calc_errors(const Space& S, const double* sol, const double* u_qp, const double* gu_qp, double* l2, double* h1);
void calc_density(const Space& S, const double* states, int k, const double* occ, double* out);
double calc_density_l2_difference(const Space& S, const double* u, const double* v, int k, const double* occ);
void calc_interpolation(const Space& S, const FaceBases& FB, const double* u_v, const double* u_e,
                        const double* u_f, const double* u_qp, double* out);

}  // namespace tsem_oracle
