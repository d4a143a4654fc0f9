// Discretisation helpers on the device: rhs, boundary conditions, errors.
#pragma once
#include <vector>

#include "common.hpp"
#include "space.hpp"

namespace tsem {

// 1-D / 2-D bases of the boundary projections (src/BuildSpace.cpp:53-170)
struct FaceBasesHost {
    int nq1 = 0, nq2 = 0, ndE = 0, ndF = 0;
    std::vector<double> interp1, face_val, interp2, add0, add1;
    void build(const SpaceHost& h, const Quadrature& Q);
};

struct PhysicsDevice {
    bool ready = false, faces_ready = false;
    DBuf<double> phi, gphi;                    // [nq3][n_loc], [nq3][n_loc][3]
    DBuf<float2> pair2;                        // [nq3][pairs a <= c] phi_a phi_c as FP32 (hi, lo) pairs
    FaceBasesHost fb;
    DBuf<double> interp1, face_val, interp2, add0, add1, b2, w2, x1, w1;
    DBuf<int> face_node, face_edge, edge_node, vdof, edof, fdof, mark_v, mark_e, mark_f;
    DBuf<uint8_t> face_same;
};

}  // namespace tsem
