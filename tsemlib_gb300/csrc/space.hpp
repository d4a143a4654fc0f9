// The TSEM space on a tetrahedral mesh: geometry information, global DOF numbering
// and the per-element global -> local transforms, built on the host once per
// (mesh, order) and mirrored to the device.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "basis.hpp"

namespace tsem {

struct MeshInput {
    int nv = 0, ne = 0, nf = 0, nt = 0;
    const double* xyz = nullptr;
    const int *edge_v = nullptr, *face_v = nullptr, *face_e = nullptr, *tet_v = nullptr, *tet_f = nullptr;
    const int *mark_v = nullptr, *mark_e = nullptr, *mark_f = nullptr;
    const int *femdof_v = nullptr, *femdof_e = nullptr;
};

struct SpaceHost {
    int M = 0, n_loc = 0, ndE = 0, ndF = 0, ndI = 0;
    int nv = 0, ne = 0, nf = 0, nt = 0;
    int64_t n_dof = 0;
    std::vector<double> xyz;
    std::vector<int> mark_v, mark_e, mark_f;
    // geometry information (src/BuildSpace.cpp:471-646)
    std::vector<int> ele_node, ele_edge, ele_face;        // [E][4], [E][6], [E][4]
    std::vector<int8_t> type_edge, type_face, type_face_inv;
    std::vector<int> edge_node, face_node, face_edge;      // [ne][2], [nf][3], [nf][3]
    std::vector<uint8_t> face_same;                        // [nf][3]
    std::vector<double> volume;                            // |T|
    // numbering (src/BuildSpace.cpp:895-948)
    std::vector<int> location_geometry, location_actualdof;
    std::vector<int> vdof, edof, fdof, tdof;               // first DOF of every geometry
    // transform global -> local, padded to max_dep terms per local index
    int max_dep = 1;
    std::vector<int> t_n, t_ind;                           // [E][n_loc], [E][n_loc][max_dep]
    std::vector<double> t_val;
    // polynomial degree of every DOF (src/Miscellaneous.cpp:557-587)
    std::vector<int> sum_dof;
    LocalTransform lt;
    StructPatterns pat;
    FaceTable ftab;

    // throws std::invalid_argument on inconsistent input
    void build(const MeshInput& in, int M);
    void closure(int e, int* out) const;     // the n_loc global DOFs of element e
};

// Candidate columns for the CSR pattern: rows on a geometry can only couple to the
// DOFs of the elements around that geometry.  cand holds one sorted list per
// geometry; row i uses list cand_geo[i].
struct PatternCandidates {
    std::vector<int64_t> geo_start;   // [n_geo_total + 1]
    std::vector<int> cand;            // concatenated sorted lists
    std::vector<int> row_geo;         // [n_dof] geometry list index of every row
    void build(const SpaceHost& S);
};

}  // namespace tsem
