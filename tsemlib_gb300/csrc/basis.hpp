// Host-side tables that define the TSEM discretisation for a polynomial order M.
#pragma once
#include <array>
#include <cstdint>
#include <vector>

namespace tsem {

int mi_count(int deg);                       // #{alpha in N^3 : |alpha| <= deg}
std::array<int, 3> mi_index(int number);     // inverse of mi_number

// phi_{target} += weight * J_alpha : the recombination of src/BuildSpace.cpp:296-413,
// stored per alpha (CSR over alpha).
struct LocalTransform {
    int M = 0, n_loc = 0;
    std::vector<int> start, target;
    std::vector<double> weight;
    void build(int M);
};

// Structural n_loc x n_loc patterns of the reference-element matrices in the
// actual basis.  These follow TSEMLib's index-offset rules exactly (mass:
// src/Discretize.cpp:126-135, stiffness: :855-883, variations :1178-1221,
// transform :1230-1244 and :435-446); deal.II keeps every diagonal.
struct StructPatterns {
    int n_loc = 0;
    std::vector<uint8_t> mass;        // [n_loc * n_loc]
    std::vector<uint8_t> stiff[6];
    std::vector<uint8_t> stiff_union;
    void build(const LocalTransform& lt);
};

// Collapsed Gauss rules on the unit interval / triangle / tetrahedron with q
// points per direction, weights normalised to unit measure (the construction of
// src/QuadInfo.cpp:63-119).
struct Quadrature {
    int q = 0;
    std::vector<double> x1, w1;       // [q]
    std::vector<double> b2, w2;       // [q*q][3] barycentric (x, y, 1-x-y)
    std::vector<double> x3, w3;       // [q^3][3]
    void build(int q);
};

// Re-expression of the face modes under the six vertex permutations of a face,
// derived here by matching traces (the reference reads the same coefficients from
// include/quad_info/Info_Interpolate_More, src/BuildSpace.cpp:1704-1771).
// Indexed like the reference: [var][local face dof] -> edge terms (edge k of the
// global face, edge dof idx, value) and face terms (face dof idx, value).
struct FaceTable {
    int M = 0, nf = 0;
    struct Edge { int k, idx; double v; };
    struct Face { int idx; double v; };
    std::vector<std::vector<std::vector<Edge>>> edge;   // [6][nf]
    std::vector<std::vector<std::vector<Face>>> face;   // [6][nf]
    void derive(int M);
};

int face_dof_index(int l1, int l2);          // (l1+l2-2)(l1+l2-3)/2 + l2-1

}  // namespace tsem
