// Right-hand sides, boundary conditions and error norms on the GPU.
//
// rhs: src/Discretize.cpp:1397-1418.  Neumann: :2011-2063.  Dirichlet: :1683-1776
// (vertex values, then edge and face values by modal projection against the
// interpolation bases, then symmetric elimination).  The elimination is written
// in gather form: a row outside the Dirichlet set subtracts A_ij u_j over its
// Dirichlet columns j, a Dirichlet row gets A_ii u_i, and the coupling entries
// are zeroed -- the same final state the reference's row-by-row loop reaches,
// because an entry is only zeroed after it has been read.  Without the matrix
// modified (modify = false) the right-hand side is formed the same way and the
// matrix is left as it is: on a matrix whose couplings are already zero that is the
// reference's result too; on one that still has them the reference's loop
// (:1752-1773) leaves an order-dependent right-hand side, which none of its drivers
// asks for.  Errors: src/CalcError.cpp.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <mutex>
#include <vector>

#include "device.hpp"
#include "jacobi.cuh"
#include "linalg.cuh"
#include "physics.hpp"

namespace tsem {

constexpr int kMaxOrderP = 16;

__global__ void k_qpoints(int E, int nq, const double* __restrict__ xyz, const int* __restrict__ nodes,
                          const double* __restrict__ x3, double* out) {
    const int64_t total = (int64_t)E * nq;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t / nq), q = (int)(t % nq);
        const double* r = x3 + 3 * (size_t)q;
        const int* nd = nodes + 4 * (size_t)e;
        for (int j = 0; j < 3; ++j) {
            const double p0 = xyz[3 * (size_t)nd[0] + j];
            out[3 * t + j] = p0 + r[0] * (xyz[3 * (size_t)nd[1] + j] - p0) + r[1] * (xyz[3 * (size_t)nd[2] + j] - p0) +
                             r[2] * (xyz[3 * (size_t)nd[3] + j] - p0);
        }
    }
}

// basis values / reference gradients at the space's 3-D quadrature points
__global__ void k_space_basis(int M, int n, int nq, const double* __restrict__ pts, const int* __restrict__ ts,
                              const int* __restrict__ tt, const double* __restrict__ tw, double* out_v, double* out_g,
                              Dual* scratch) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    Dual* J = scratch + (size_t)q * n;
    const Dual x(pts[3 * q], 1, 0, 0), y(pts[3 * q + 1], 0, 1, 0), z(pts[3 * q + 2], 0, 0, 1);
    jacobi_products<Dual, kMaxOrderP>(M, x, y, z, J);
    for (int i = 0; i < n; ++i) {
        out_v[(size_t)q * n + i] = 0;
        for (int d = 0; d < 3; ++d) out_g[((size_t)q * n + i) * 3 + d] = 0;
    }
    for (int a = 0; a < n; ++a)
        for (int j = ts[a]; j < ts[a + 1]; ++j) {
            const int t = tt[j];
            const double w = tw[j];
            out_v[(size_t)q * n + t] += w * J[a].v;
            out_g[((size_t)q * n + t) * 3 + 0] += w * J[a].d0;
            out_g[((size_t)q * n + t) * 3 + 1] += w * J[a].d1;
            out_g[((size_t)q * n + t) * 3 + 2] += w * J[a].d2;
        }
}

void physics_basis(tsem_space_s* sp) {
    space_upload(sp);
    auto& P = sp->phys;
    if (P.ready) return;
    auto& h = sp->host;
    cudaStream_t s = sp->stream;
    const int nq = (int)sp->quad.w3.size(), n = h.n_loc;
    DBuf<int> ts, tt;
    DBuf<double> tw;
    DBuf<Dual> scratch((size_t)nq * n);
    ts.upload(h.lt.start, s);
    tt.upload(h.lt.target, s);
    tw.upload(h.lt.weight, s);
    P.phi.alloc((size_t)nq * n);
    P.gphi.alloc((size_t)nq * n * 3);
    k_space_basis<<<(nq + 63) / 64, 64, 0, s>>>(h.M, n, nq, sp->dev.x3.p, ts.p, tt.p, tw.p, P.phi.p, P.gphi.p, scratch.p);
    TSEM_LAUNCHED();
    TSEM_CUDA(cudaStreamSynchronize(s));
    P.ready = true;
}

void element_qpoints(tsem_space_s* sp, double* host_out) {
    space_upload(sp);
    auto& h = sp->host;
    cudaStream_t s = sp->stream;
    const int nq = (int)sp->quad.w3.size();
    DBuf<double> out((size_t)h.nt * nq * 3);
    k_qpoints<<<grid_for((int64_t)h.nt * nq, 256), 256, 0, s>>>(h.nt, nq, sp->dev.xyz.p, sp->dev.ele_node.p, sp->dev.x3.p, out.p);
    TSEM_LAUNCHED();
    out.download(host_out, out.n, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
}

// ------------------------------------------------------------------------ rhs
// b_i += |T| sum_q w_q f_q phi_i(q) scattered through the transform; one block per element
__global__ void k_rhs(int n_loc, int nq, int max_dep, const double* __restrict__ f, const double* __restrict__ w,
                      const double* __restrict__ phi, const double* __restrict__ vol, const int* __restrict__ t_n,
                      const int* __restrict__ t_ind, const double* __restrict__ t_val, double* rhs) {
    const int e = blockIdx.x;
    const double* fe = f + (size_t)e * nq;   // the same point for every thread: broadcast loads
    for (int i = threadIdx.x; i < n_loc; i += blockDim.x) {
        double c = 0;
        for (int q = 0; q < nq; ++q) {
            const double wf = w[q] * fe[q];
            c += wf * phi[(size_t)q * n_loc + i];
        }
        c *= vol[e];
        const size_t b = (size_t)e * n_loc + i;
        for (int j = 0; j < t_n[b]; ++j) atomicAdd(rhs + t_ind[b * max_dep + j], c * t_val[b * max_dep + j]);
    }
}

// device arrays, enqueued on s
void rhs_device(tsem_space_s* sp, const double* f_qp, double* out, cudaStream_t s) {
    physics_basis(sp);
    TSEM_CUDA(cudaStreamSynchronize(sp->stream));   // the space's device data is in place
    auto& h = sp->host;
    const int nq = (int)sp->quad.w3.size();
    TSEM_CUDA(cudaMemsetAsync(out, 0, (size_t)h.n_dof * sizeof(double), s));
    k_rhs<<<h.nt, 128, 0, s>>>(h.n_loc, nq, h.max_dep, f_qp, sp->dev.w3.p, sp->phys.phi.p,
                                                 sp->dev.volume.p, sp->dev.t_n.p, sp->dev.t_ind.p, sp->dev.t_val.p, out);
    TSEM_LAUNCHED();
}

void rhs(tsem_space_s* sp, const double* f_qp_host, double* rhs_host) {
    physics_basis(sp);
    auto& h = sp->host;
    cudaStream_t s = sp->stream;
    const int nq = (int)sp->quad.w3.size();
    DBuf<double> f, out(h.n_dof);
    f.upload(f_qp_host, (size_t)h.nt * nq, s);
    rhs_device(sp, f.p, out.p, s);
    out.download(rhs_host, h.n_dof, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
}

// ------------------------------------------------------------------ face bases
void FaceBasesHost::build(const SpaceHost& h, const Quadrature& Q) {
    const int M = h.M;
    nq1 = (int)Q.w1.size();
    nq2 = (int)Q.w2.size();
    ndE = h.ndE;
    ndF = h.ndF;
    interp1.assign((size_t)nq1 * std::max(ndE, 1), 0.0);
    face_val.assign((size_t)nq2 * std::max(ndF, 1), 0.0);
    interp2.assign((size_t)nq2 * std::max(ndF, 1), 0.0);
    add0.assign((size_t)nq2 * std::max(ndE, 1), 0.0);
    add1.assign((size_t)nq2 * std::max(ndE, 1), 0.0);
    std::vector<double> P(M + 2), P2(M + 2), J(M + 2), Je(M + 2);
    for (int p = 0; p < nq1; ++p) {
        jacobi_classic<double>(1, 1, 2 * Q.x1[p] - 1, std::max(M - 2, 0), P.data());
        for (int l = 0; l < ndE; ++l) interp1[(size_t)p * ndE + l] = P[l];
    }
    for (int p = 0; p < nq2; ++p) {
        const double x = Q.b2[3 * p], y = Q.b2[3 * p + 1];
        const double xi = 2 * x / (1 - y) - 1, eta = 2 * y - 1;
        jacobi_general<double, 64>(-1, -1, xi, M, J.data());
        for (int l1 = 2; l1 <= M; ++l1) {
            jacobi_general<double, 64>(2 * l1 - 1, -1, eta, M - l1, Je.data());
            for (int l2 = 1; l2 <= M - l1; ++l2)
                face_val[(size_t)p * ndF + face_dof_index(l1, l2)] = 2 * std::pow(1 - y, l1) * J[l1] * Je[l2];
        }
        jacobi_classic<double>(1, 1, xi, std::max(M - 2, 0), P.data());
        for (int l1 = 2; l1 <= M; ++l1) {
            jacobi_classic<double>(2 * l1 - 1, 1, eta, std::max(M - l1 - 1, 0), P2.data());
            for (int l2 = 1; l2 <= M - l1; ++l2)
                interp2[(size_t)p * ndF + face_dof_index(l1, l2)] = std::pow(1 - eta, l1 - 2) * P[l1 - 2] * P2[l2 - 1];
        }
        jacobi_classic<double>(1, 1, eta, std::max(M - 2, 0), P2.data());
        for (int l = 2; l <= M; ++l) {
            add0[(size_t)p * ndE + l - 2] = std::pow(1 - y, l - 2) * P[l - 2];
            add1[(size_t)p * ndE + l - 2] = P2[l - 2];
        }
    }
}

void physics_faces(tsem_space_s* sp) {
    space_upload(sp);
    auto& F = sp->phys;
    if (F.faces_ready) return;
    cudaStream_t s = sp->stream;
    F.fb.build(sp->host, sp->quad);
    F.interp1.upload(F.fb.interp1, s);
    F.face_val.upload(F.fb.face_val, s);
    F.interp2.upload(F.fb.interp2, s);
    F.add0.upload(F.fb.add0, s);
    F.add1.upload(F.fb.add1, s);
    F.b2.upload(sp->quad.b2, s);
    F.w2.upload(sp->quad.w2, s);
    F.x1.upload(sp->quad.x1, s);
    F.w1.upload(sp->quad.w1, s);
    auto& h = sp->host;
    F.face_node.upload(h.face_node, s);
    F.face_edge.upload(h.face_edge, s);
    F.face_same.upload(h.face_same, s);
    F.edge_node.upload(h.edge_node, s);
    F.vdof.upload(h.vdof, s);
    F.edof.upload(h.edof, s);
    F.fdof.upload(h.fdof, s);
    F.mark_v.upload(h.mark_v, s);
    F.mark_e.upload(h.mark_e, s);
    F.mark_f.upload(h.mark_f, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    F.faces_ready = true;
}

void boundary_points(tsem_space_s* sp, int dim, double* out, int64_t* count) {
    auto& h = sp->host;
    const Quadrature& Q = sp->quad;
    const int nq1 = (int)Q.w1.size(), nq2 = (int)Q.w2.size();
    if (dim == 0) {
        *count = h.nv;
        if (out) std::copy(h.xyz.begin(), h.xyz.end(), out);
    } else if (dim == 1) {
        *count = (int64_t)h.ne * nq1;
        if (out)
            for (int g = 0; g < h.ne; ++g)
                for (int p = 0; p < nq1; ++p)
                    for (int j = 0; j < 3; ++j)
                        out[((size_t)g * nq1 + p) * 3 + j] = h.xyz[3 * (size_t)h.edge_node[2 * g] + j] * (1 - Q.x1[p]) +
                                                              h.xyz[3 * (size_t)h.edge_node[2 * g + 1] + j] * Q.x1[p];
    } else {
        *count = (int64_t)h.nf * nq2;
        if (out)
            for (int f = 0; f < h.nf; ++f)
                for (int p = 0; p < nq2; ++p)
                    for (int j = 0; j < 3; ++j) {
                        double v = 0;
                        for (int k = 0; k < 3; ++k) v += h.xyz[3 * (size_t)h.face_node[3 * f + k] + j] * Q.b2[3 * p + (k + 2) % 3];
                        out[((size_t)f * nq2 + p) * 3 + j] = v;
                    }
    }
}

// -------------------------------------------------------------------- Neumann
__global__ void k_neumann(int nf, int nq2, int ndE, int ndF, int flag, const int* __restrict__ mark_f,
                          const double* __restrict__ g, const double* __restrict__ xyz, const int* __restrict__ face_node,
                          const int* __restrict__ face_edge, const uint8_t* __restrict__ face_same,
                          const double* __restrict__ b2, const double* __restrict__ w2, const double* __restrict__ add0,
                          const double* __restrict__ add1, const double* __restrict__ face_val, const int* __restrict__ vdof,
                          const int* __restrict__ edof, const int* __restrict__ fdof, double* rhs) {
    const int f = blockIdx.x;
    if (f >= nf || mark_f[f] != flag) return;
    const double* p0 = xyz + 3 * (size_t)face_node[3 * f];
    const double* p1 = xyz + 3 * (size_t)face_node[3 * f + 1];
    const double* p2 = xyz + 3 * (size_t)face_node[3 * f + 2];
    const double c0 = (p1[1] - p0[1]) * (p2[2] - p0[2]) - (p1[2] - p0[2]) * (p2[1] - p0[1]);
    const double c1 = (p1[0] - p0[0]) * (p2[2] - p0[2]) - (p1[2] - p0[2]) * (p2[0] - p0[0]);
    const double c2 = (p1[0] - p0[0]) * (p2[1] - p0[1]) - (p1[1] - p0[1]) * (p2[0] - p0[0]);
    const double area = 0.5 * sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    // one thread per output: 3 vertex terms, 3*ndE edge terms, ndF face terms
    const int nout = 3 + 3 * ndE + ndF;
    for (int o = threadIdx.x; o < nout; o += blockDim.x) {
        double acc = 0;
        for (int p = 0; p < nq2; ++p) {
            const double x = b2[3 * p], y = b2[3 * p + 1], r = b2[3 * p + 2];
            const double wgv = w2[p] * g[(size_t)f * nq2 + p] * area;
            double basis;
            if (o < 3) {
                basis = b2[3 * p + (o + 2) % 3];
            } else if (o < 3 + 3 * ndE) {
                const int k = (o - 3) / ndE, i = (o - 3) % ndE;
                basis = k == 0 ? -2 * x * y * add1[(size_t)p * ndE + i]
                               : (k == 1 ? -2 * y * r * add1[(size_t)p * ndE + i] : -2 * x * r * add0[(size_t)p * ndE + i]);
            } else {
                basis = face_val[(size_t)p * ndF + (o - 3 - 3 * ndE)];
            }
            acc += wgv * basis;
        }
        if (o < 3) {
            atomicAdd(rhs + vdof[face_node[3 * f + o]], acc);
        } else if (o < 3 + 3 * ndE) {
            const int k = (o - 3) / ndE, i = (o - 3) % ndE;
            if (!face_same[3 * f + k] && (i & 1)) acc = -acc;
            atomicAdd(rhs + edof[face_edge[3 * f + k]] + i, acc);
        } else {
            atomicAdd(rhs + fdof[f] + (o - 3 - 3 * ndE), acc);
        }
    }
}

void neumann(tsem_space_s* sp, double* rhs_host, const double* g_host, int flag) {
    physics_faces(sp);
    auto& h = sp->host;
    auto& F = sp->phys;
    cudaStream_t s = sp->stream;
    DBuf<double> g, r;
    g.upload(g_host, (size_t)h.nf * F.fb.nq2, s);
    r.upload(rhs_host, h.n_dof, s);
    k_neumann<<<h.nf, 128, 0, s>>>(h.nf, F.fb.nq2, h.ndE, h.ndF, flag, F.mark_f.p, g.p, sp->dev.xyz.p, F.face_node.p,
                                   F.face_edge.p, F.face_same.p, F.b2.p, F.w2.p, F.add0.p, F.add1.p, F.face_val.p, F.vdof.p,
                                   F.edof.p, F.fdof.p, r.p);
    TSEM_LAUNCHED();
    r.download(rhs_host, h.n_dof, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
}

// ------------------------------------------------------------------ Dirichlet
__global__ void k_dir_vertex(int nv, int flag, const int* __restrict__ mark_v, const double* __restrict__ u,
                             const int* __restrict__ vdof, double* val, uint8_t* isd) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        const bool on = flag == -2 || (flag == -1 ? mark_v[v] != 0 : mark_v[v] == flag);
        if (!on) continue;
        val[vdof[v]] = u[v];
        isd[vdof[v]] = 1;
    }
}

// edge modal values: c_l = -l(2l-1)/(2(l-1)) sum_p w_p (u - u_s(1-x) - u_e x) P_{l-2}^{1,1}(2x-1)
__global__ void k_dir_edge(int ne, int nq1, int ndE, int flag, const int* __restrict__ mark_e, const double* __restrict__ u,
                           const int* __restrict__ edge_node, const int* __restrict__ vdof, const int* __restrict__ edof,
                           const double* __restrict__ x1, const double* __restrict__ w1, const double* __restrict__ interp1,
                           double* val, uint8_t* isd) {
    const int64_t total = (int64_t)ne * ndE;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)(t / ndE), i = (int)(t % ndE);
        const bool on = flag == -2 || (flag == -1 ? mark_e[g] != 0 : mark_e[g] == flag);
        if (!on) continue;
        const double cs = val[vdof[edge_node[2 * g]]], ce = val[vdof[edge_node[2 * g + 1]]];
        double c = 0;
        for (int p = 0; p < nq1; ++p)
            c += w1[p] * (u[(size_t)g * nq1 + p] - cs * (1 - x1[p]) - ce * x1[p]) * interp1[(size_t)p * ndE + i];
        const int l = i + 2;
        val[edof[g] + i] = c * -l * (2 * l - 1) / (2.0 * (l - 1));
        isd[edof[g] + i] = 1;
    }
}

__global__ void k_dir_face(int nf, int nq2, int ndE, int ndF, int M, int flag, const int* __restrict__ mark_f,
                           const double* __restrict__ u, const int* __restrict__ face_node, const int* __restrict__ face_edge,
                           const uint8_t* __restrict__ face_same, const int* __restrict__ vdof, const int* __restrict__ edof,
                           const int* __restrict__ fdof, const double* __restrict__ b2, const double* __restrict__ w2,
                           const double* __restrict__ add0, const double* __restrict__ add1,
                           const double* __restrict__ interp2, double* val, uint8_t* isd) {
    const int64_t total = (int64_t)nf * ndF;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int f = (int)(t / ndF), di = (int)(t % ndF);
        const bool on = flag == -2 || (flag == -1 ? mark_f[f] != 0 : mark_f[f] == flag);
        if (!on) continue;
        double vv[3];
        for (int k = 0; k < 3; ++k) vv[k] = val[vdof[face_node[3 * f + k]]];
        int l1 = 2, l2 = 1;
        for (int a = 2; a <= M; ++a)
            for (int b = 1; b <= M - a; ++b)
                if ((a + b - 2) * (a + b - 3) / 2 + b - 1 == di) { l1 = a; l2 = b; }
        double c = 0;
        for (int p = 0; p < nq2; ++p) {
            const double xp = b2[3 * p], yp = b2[3 * p + 1], rp = b2[3 * p + 2];
            double cp = u[(size_t)f * nq2 + p];
            for (int k = 0; k < 3; ++k) cp -= vv[k] * b2[3 * p + (k + 2) % 3];
            for (int k = 0; k < 3; ++k) {
                const int e0 = edof[face_edge[3 * f + k]];
                const bool same = face_same[3 * f + k];
                for (int i = 0; i < ndE; ++i) {
                    double ev = val[e0 + i];
                    if (!same && ((i + 2) & 1)) ev = -ev;
                    const double tr = k == 0 ? xp * yp * add1[(size_t)p * ndE + i]
                                             : (k == 1 ? yp * rp * add1[(size_t)p * ndE + i] : xp * rp * add0[(size_t)p * ndE + i]);
                    cp += 2 * ev * tr;
                }
            }
            c += w2[p] * cp * interp2[(size_t)p * ndF + di];
        }
        val[fdof[f] + di] = c * -l1 * (2 * l1 - 1) * (2 * l1 + 2 * l2 - 1) / (pow(2.0, l1) * (l1 - 1));
        isd[fdof[f] + di] = 1;
    }
}

// gather-form elimination: see the file comment
__global__ void k_dir_rhs(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ ci,
                          const double* __restrict__ va, const uint8_t* __restrict__ isd, const double* __restrict__ val,
                          double* rhs) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        if (isd[r]) {
            rhs[r] = va[rp[r]] * val[r];
            continue;
        }
        double s = 0;
        for (int64_t k = rp[r] + 1; k < rp[r + 1]; ++k)
            if (isd[ci[k]]) s += va[k] * val[ci[k]];
        rhs[r] -= s;
    }
}

__global__ void k_zero_couplings(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ ci,
                                 const uint8_t* __restrict__ isd, double* va) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const bool rd = isd[r];
        for (int64_t k = rp[r] + 1; k < rp[r + 1]; ++k)
            if (rd || isd[ci[k]]) va[k] = 0.0;
    }
}

static void check_closure(const SpaceHost& h, int flag) {
    auto on = [&](int m) { return flag == -1 ? m != 0 : m == flag; };
    for (int f = 0; f < h.nf; ++f) {
        if (!on(h.mark_f[f])) continue;
        for (int k = 0; k < 3; ++k)
            if (!on(h.mark_e[h.face_edge[3 * f + k]]) || !on(h.mark_v[h.face_node[3 * f + k]]))
                throw Error(TSEM_INVALID, "a Dirichlet face has an edge or vertex outside the Dirichlet set");
    }
    for (int e = 0; e < h.ne; ++e) {
        if (!on(h.mark_e[e])) continue;
        if (!on(h.mark_v[h.edge_node[2 * e]]) || !on(h.mark_v[h.edge_node[2 * e + 1]]))
            throw Error(TSEM_INVALID, "a Dirichlet edge has a vertex outside the Dirichlet set");
    }
}

void dirichlet(tsem_space_s* sp, DevCsr& A, double* rhs_host, const double* uv, const double* ue, const double* uf,
               bool modify, int flag) {
    physics_faces(sp);
    auto& h = sp->host;
    auto& F = sp->phys;
    cudaStream_t s = sp->stream;
    if (A.n != h.n_dof) throw Error(TSEM_INVALID, "matrix size differs from the space");
    check_closure(h, flag);
    DBuf<double> du_v, du_e, du_f, val(h.n_dof), r;
    DBuf<uint8_t> isd(h.n_dof);
    du_v.upload(uv, h.nv, s);
    du_e.upload(ue, (size_t)h.ne * F.fb.nq1, s);
    du_f.upload(uf, (size_t)h.nf * F.fb.nq2, s);
    r.upload(rhs_host, h.n_dof, s);
    val.zero(s);
    isd.zero(s);
    k_dir_vertex<<<grid_for(h.nv, 256), 256, 0, s>>>(h.nv, flag, F.mark_v.p, du_v.p, F.vdof.p, val.p, isd.p);
    TSEM_LAUNCHED();
    if (h.ndE > 0)
        k_dir_edge<<<grid_for((int64_t)h.ne * h.ndE, 256), 256, 0, s>>>(h.ne, F.fb.nq1, h.ndE, flag, F.mark_e.p, du_e.p,
                                                                       F.edge_node.p, F.vdof.p, F.edof.p, F.x1.p, F.w1.p,
                                                                       F.interp1.p, val.p, isd.p);
        TSEM_LAUNCHED();
    if (h.ndF > 0)
        k_dir_face<<<grid_for((int64_t)h.nf * h.ndF, 128), 128, 0, s>>>(h.nf, F.fb.nq2, h.ndE, h.ndF, h.M, flag, F.mark_f.p,
                                                                       du_f.p, F.face_node.p, F.face_edge.p, F.face_same.p,
                                                                       F.vdof.p, F.edof.p, F.fdof.p, F.b2.p, F.w2.p, F.add0.p,
                                                                       F.add1.p, F.interp2.p, val.p, isd.p);
    TSEM_LAUNCHED();
    k_dir_rhs<<<grid_for(h.n_dof, 256), 256, 0, s>>>(h.n_dof, A.rowptr.p, A.col.p, A.val.p, isd.p, val.p, r.p);
    TSEM_LAUNCHED();
    if (modify) {
        k_zero_couplings<<<grid_for(h.n_dof, 256), 256, 0, s>>>(h.n_dof, A.rowptr.p, A.col.p, isd.p, A.val.p);
        TSEM_LAUNCHED();
        A.values_changed();
    }
    r.download(rhs_host, h.n_dof, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
}

__global__ void k_mark_dofs(int nv, int ne, int nf, int ndE, int ndF, int flag, const int* __restrict__ mv,
                            const int* __restrict__ me, const int* __restrict__ mf, const int* __restrict__ vdof,
                            const int* __restrict__ edof, const int* __restrict__ fdof, uint8_t* isd) {
    const int64_t total = (int64_t)nv + ne + nf;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        if (t < nv) {
            if (mv[t] == flag) isd[vdof[t]] = 1;
        } else if (t < nv + ne) {
            const int e = (int)(t - nv);
            if (me[e] == flag)
                for (int i = 0; i < ndE; ++i) isd[edof[e] + i] = 1;
        } else {
            const int f = (int)(t - nv - ne);
            if (mf[f] == flag)
                for (int i = 0; i < ndF; ++i) isd[fdof[f] + i] = 1;
        }
    }
}

__global__ void k_zero_rows(int64_t n, const uint8_t* __restrict__ isd, double* rhs) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        if (isd[r]) rhs[r] = 0.0;
}

void zero_bc(tsem_space_s* sp, DevCsr* A, double* rhs_host, int flag) {
    physics_faces(sp);
    auto& h = sp->host;
    auto& F = sp->phys;
    cudaStream_t s = sp->stream;
    DBuf<uint8_t> isd(h.n_dof);
    isd.zero(s);
    k_mark_dofs<<<grid_for((int64_t)h.nv + h.ne + h.nf, 256), 256, 0, s>>>(h.nv, h.ne, h.nf, h.ndE, h.ndF, flag, F.mark_v.p,
                                                                          F.mark_e.p, F.mark_f.p, F.vdof.p, F.edof.p,
                                                                          F.fdof.p, isd.p);
    TSEM_LAUNCHED();
    if (A) {
        if (A->n != h.n_dof) throw Error(TSEM_INVALID, "matrix size differs from the space");
        k_zero_couplings<<<grid_for(h.n_dof, 256), 256, 0, s>>>(h.n_dof, A->rowptr.p, A->col.p, isd.p, A->val.p);
        A->values_changed();
        TSEM_LAUNCHED();
    }
    if (rhs_host) {
        DBuf<double> r;
        r.upload(rhs_host, h.n_dof, s);
        k_zero_rows<<<grid_for(h.n_dof, 256), 256, 0, s>>>(h.n_dof, isd.p, r.p);
        TSEM_LAUNCHED();
        r.download(rhs_host, h.n_dof, s);
    }
    TSEM_CUDA(cudaStreamSynchronize(s));
}

// ------------------------------------------------------------------- errors
__global__ void k_errors(int n_loc, int nq, int max_dep, const double* __restrict__ sol, const double* __restrict__ uq,
                         const double* __restrict__ guq, const double* __restrict__ w, const double* __restrict__ phi,
                         const double* __restrict__ gphi, const double* __restrict__ xyz, const int* __restrict__ nodes,
                         const double* __restrict__ vol, const int* __restrict__ t_n, const int* __restrict__ t_ind,
                         const double* __restrict__ t_val, double* out) {
    const int e = blockIdx.x;
    extern __shared__ double c[];
    for (int i = threadIdx.x; i < n_loc; i += blockDim.x) {
        const size_t b = (size_t)e * n_loc + i;
        double s = 0;
        for (int j = 0; j < t_n[b]; ++j) s += sol[t_ind[b * max_dep + j]] * t_val[b * max_dep + j];
        c[i] = s;
    }
    __shared__ double Ji[3][3];
    if (threadIdx.x == 0) {
        const int* nd = nodes + 4 * (size_t)e;
        double d[3][3];
        for (int k = 0; k < 3; ++k)
            for (int j = 0; j < 3; ++j) d[j][k] = xyz[3 * (size_t)nd[k + 1] + j] - xyz[3 * (size_t)nd[0] + j];
        const double V = d[0][0] * d[1][1] * d[2][2] + d[0][1] * d[1][2] * d[2][0] + d[0][2] * d[1][0] * d[2][1] -
                         d[0][0] * d[1][2] * d[2][1] - d[0][1] * d[1][0] * d[2][2] - d[0][2] * d[1][1] * d[2][0];
        Ji[0][0] = (d[1][1] * d[2][2] - d[1][2] * d[2][1]) / V;
        Ji[0][1] = (d[0][2] * d[2][1] - d[0][1] * d[2][2]) / V;
        Ji[0][2] = (d[0][1] * d[1][2] - d[0][2] * d[1][1]) / V;
        Ji[1][0] = (d[1][2] * d[2][0] - d[1][0] * d[2][2]) / V;
        Ji[1][1] = (d[0][0] * d[2][2] - d[0][2] * d[2][0]) / V;
        Ji[1][2] = (d[0][2] * d[1][0] - d[0][0] * d[1][2]) / V;
        Ji[2][0] = (d[1][0] * d[2][1] - d[1][1] * d[2][0]) / V;
        Ji[2][1] = (d[0][1] * d[2][0] - d[0][0] * d[2][1]) / V;
        Ji[2][2] = (d[0][0] * d[1][1] - d[0][1] * d[1][0]) / V;
    }
    __syncthreads();
    double acc[2] = {0, 0};
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        double v = 0, gr[3] = {0, 0, 0};
        for (int i = 0; i < n_loc; ++i) {
            v += c[i] * phi[(size_t)q * n_loc + i];
            const double* g = gphi + ((size_t)q * n_loc + i) * 3;
            for (int k = 0; k < 3; ++k) gr[k] += c[i] * (Ji[0][k] * g[0] + Ji[1][k] * g[1] + Ji[2][k] * g[2]);
        }
        const size_t eq = (size_t)e * nq + q;
        const double du = v - uq[eq];
        double dg = 0;
        for (int k = 0; k < 3; ++k) dg += (gr[k] - guq[3 * eq + k]) * (gr[k] - guq[3 * eq + k]);
        acc[0] += w[q] * du * du * vol[e];
        acc[1] += w[q] * dg * vol[e];
    }
    double* const dst[2] = {out, out + 1};
    block_accumulate<2>(acc, dst);
}

void errors(tsem_space_s* sp, const double* sol_host, const double* uq_host, const double* guq_host, double* out) {
    physics_basis(sp);
    auto& h = sp->host;
    cudaStream_t s = sp->stream;
    const int nq = (int)sp->quad.w3.size();
    DBuf<double> sol, uq, guq, acc(2);
    sol.upload(sol_host, h.n_dof, s);
    uq.upload(uq_host, (size_t)h.nt * nq, s);
    guq.upload(guq_host, (size_t)h.nt * nq * 3, s);
    acc.zero(s);
    k_errors<<<h.nt, 128, h.n_loc * sizeof(double), s>>>(h.n_loc, nq, h.max_dep, sol.p, uq.p, guq.p, sp->dev.w3.p,
                                                         sp->phys.phi.p, sp->phys.gphi.p, sp->dev.xyz.p, sp->dev.ele_node.p,
                                                         sp->dev.volume.p, sp->dev.t_n.p, sp->dev.t_ind.p, sp->dev.t_val.p,
                                                         acc.p);
    TSEM_LAUNCHED();
    double hh[2];
    acc.download(hh, 2, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    out[0] = std::sqrt(hh[0]);
    out[1] = std::sqrt(hh[1]);
}

}  // namespace tsem

namespace tsem {

// ------------------------------------------------- potential matrix (mass_V)
__device__ __forceinline__ int64_t find_col(const int64_t* __restrict__ rowptr, const int* __restrict__ col, int r, int c) {
    const int64_t b = rowptr[r], e = rowptr[r + 1];
    if (col[b] == c) return b;
    int64_t lo = b + 1, hi = e;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (col[mid] < c) lo = mid + 1; else hi = mid;
    }
    return (lo < e && col[lo] == c) ? lo : -1;
}

// phi_a(q) phi_c(q) for the pairs a <= c (row-major over the upper triangle), split
// into FP32 (hi, lo) pairs: the same for every element
__global__ void k_pair_products(int n_loc, int nq, const double* __restrict__ phi, float2* __restrict__ out) {
    const int npair = n_loc * (n_loc + 1) / 2;
    const int64_t total = (int64_t)nq * npair;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(t / npair);
        int a = 0, rem = (int)(t % npair);
        while (rem >= n_loc - a) { rem -= n_loc - a; ++a; }
        const int c = a + rem;
        const double v = phi[(size_t)q * n_loc + a] * phi[(size_t)q * n_loc + c];
        const float hi = __double2float_rn(v);
        out[t] = make_float2(hi, __double2float_rn(v - (double)hi));
    }
}

// (sh, sl) += a * b for FP32 (hi, lo) pairs: exact product error by FMA, compensated sum
__device__ __forceinline__ void pot_acc2(float2 a, float2 b, float& sh, float& sl) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    const float t = __fadd_rn(sh, p);
    const float bp = __fsub_rn(t, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    sh = t;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// build_mass_V_matrix (src/Discretize.cpp:668-756): the element block
// B_e[a][c] = sum_q (w_q V_e(q) |T_e|) phi_a(q) phi_c(q) of every pair a <= c, scattered
// (with its mirror) through the transform.  The pair products are shared by all
// elements, so a block takes kPotElems elements and blockDim.x pairs: one product
// load feeds kPotElems sums.  FP64 on the FP32 pipe (split operands, compensated
// sums, about 2^-44 relative per entry); the scatter adds in FP64.
constexpr int kPotElems = 8;
__global__ void k_potential2(int E, int n_loc, int nq, int max_dep, const double* __restrict__ v,
                             const double* __restrict__ w, const float2* __restrict__ pair2,
                             const double* __restrict__ vol, const int* __restrict__ t_n, const int* __restrict__ t_ind,
                             const double* __restrict__ t_val, const int64_t* __restrict__ rowptr,
                             const int* __restrict__ col, double* val, int* err) {
    extern __shared__ float2 wv2[];   // [kPotElems][nq]
    const int e0 = blockIdx.y * kPotElems;
    for (int t = threadIdx.x; t < kPotElems * nq; t += blockDim.x) {
        const int j = t / nq, q = t % nq, e = e0 + j;
        const double x = e < E ? w[q] * v[(size_t)e * nq + q] * vol[e] : 0.0;
        const float hi = __double2float_rn(x);
        wv2[t] = make_float2(hi, __double2float_rn(x - (double)hi));
    }
    __syncthreads();
    const int npair = n_loc * (n_loc + 1) / 2;
    const int pi = blockIdx.x * blockDim.x + threadIdx.x;
    if (pi >= npair) return;
    float sh[kPotElems], sl[kPotElems];
#pragma unroll
    for (int j = 0; j < kPotElems; ++j) sh[j] = sl[j] = 0.0f;
    for (int q = 0; q < nq; ++q) {
        const float2 pq = pair2[(size_t)q * npair + pi];
#pragma unroll
        for (int j = 0; j < kPotElems; ++j) pot_acc2(wv2[j * nq + q], pq, sh[j], sl[j]);
    }
    int a = 0, rem = pi;
    while (rem >= n_loc - a) { rem -= n_loc - a; ++a; }
    const int c = a + rem;
    for (int j = 0; j < kPotElems; ++j) {
        const int e = e0 + j;
        if (e >= E) break;
        const double acc = (double)sh[j] + (double)sl[j];
        const size_t ba = (size_t)e * n_loc + a, bc = (size_t)e * n_loc + c;
        const int na = t_n[ba], nc = t_n[bc];
        for (int u = 0; u < na; ++u) {
            const int r = t_ind[ba * max_dep + u];
            const double tu = acc * t_val[ba * max_dep + u];
            for (int x = 0; x < nc; ++x) {
                const int cc = t_ind[bc * max_dep + x];
                const double vv = tu * t_val[bc * max_dep + x];
                const int64_t p1 = find_col(rowptr, col, r, cc);
                if (p1 < 0) { atomicExch(err, 1); continue; }
                atomicAdd(val + p1, vv);
                if (a != c) {
                    const int64_t p2 = find_col(rowptr, col, cc, r);
                    if (p2 < 0) { atomicExch(err, 1); continue; }
                    atomicAdd(val + p2, vv);
                }
            }
        }
    }
}


void assemble_potential(tsem_space_s* sp, const double* v_qp_host, DevCsr& A) {
    auto& h = sp->host;
    cudaStream_t s = sp->stream;
    const int nq = (int)sp->quad.w3.size();
    DBuf<double> v;
    v.upload(v_qp_host, (size_t)h.nt * nq, s);
    assemble_potential_device(sp, v.p, A, s);
}

// V at the element quadrature points in device memory, ready on stream s; returns
// after the matrix is complete
void assemble_potential_device(tsem_space_s* sp, const double* v_qp, DevCsr& A, cudaStream_t s) {
    physics_basis(sp);
    TSEM_CUDA(cudaStreamSynchronize(sp->stream));   // the space's device data is in place
    auto& h = sp->host;
    const int nq = (int)sp->quad.w3.size();
    if (A.n != h.n_dof || !A.rowptr.p) {
        TSEM_CUDA(cudaStreamSynchronize(s));
        space_pattern_full(sp, A);
        TSEM_CUDA(cudaStreamSynchronize(sp->stream));
    }
    const int npair = h.n_loc * (h.n_loc + 1) / 2;
    if (sp->phys.pair2.n != (size_t)nq * npair) {
        sp->phys.pair2.alloc((size_t)nq * npair);
        k_pair_products<<<grid_for((int64_t)nq * npair, 256), 256, 0, s>>>(h.n_loc, nq, sp->phys.phi.p, sp->phys.pair2.p);
        TSEM_LAUNCHED();
    }
    A.val.zero(s);
    DBuf<int> err(1);
    err.zero(s);
    const size_t shm = (size_t)kPotElems * nq * sizeof(float2);
    {
        static std::once_flag once;   // orders up to 8 stage 8 x 1000 points
        std::call_once(once, [] {
            TSEM_CUDA(cudaFuncSetAttribute(k_potential2, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
        });
    }
    if (shm > 160 * 1024) throw Error(TSEM_INVALID, "potential matrix: too many quadrature points per element");
    const dim3 g((unsigned)((npair + 127) / 128), (unsigned)((h.nt + kPotElems - 1) / kPotElems));
    k_potential2<<<g, 128, shm, s>>>(
        h.nt, h.n_loc, nq, h.max_dep, v_qp, sp->dev.w3.p, sp->phys.pair2.p, sp->dev.volume.p, sp->dev.t_n.p,
        sp->dev.t_ind.p, sp->dev.t_val.p, A.rowptr.p, A.col.p, A.val.p, err.p);
    TSEM_LAUNCHED();
    A.refresh_diag(s);
    A.spmv_variant = -1;
    int herr = 0;
    err.download(&herr, 1, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    if (herr) throw Error(TSEM_INVALID, "potential matrix: entry outside the pattern (matrix from another space?)");
}

// values of an FE function at the element quadrature points; one block per element
__global__ void k_eval_qp(int n_loc, int nq, int max_dep, const double* __restrict__ sol, const double* __restrict__ phi,
                          const int* __restrict__ t_n, const int* __restrict__ t_ind, const double* __restrict__ t_val,
                          double* out) {
    const int e = blockIdx.x;
    extern __shared__ double c[];
    for (int i = threadIdx.x; i < n_loc; i += blockDim.x) {
        const size_t b = (size_t)e * n_loc + i;
        double s = 0;
        for (int j = 0; j < t_n[b]; ++j) s += sol[t_ind[b * max_dep + j]] * t_val[b * max_dep + j];
        c[i] = s;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        double v = 0;
        for (int i = 0; i < n_loc; ++i) v += c[i] * phi[(size_t)q * n_loc + i];
        out[(size_t)e * nq + q] = v;
    }
}

// device arrays, enqueued on s
void eval_qp_device(tsem_space_s* sp, const double* sol, double* out, cudaStream_t s) {
    physics_basis(sp);
    TSEM_CUDA(cudaStreamSynchronize(sp->stream));   // the space's device data is in place
    auto& h = sp->host;
    const int nq = (int)sp->quad.w3.size();
    k_eval_qp<<<h.nt, 128, h.n_loc * sizeof(double), s>>>(h.n_loc, nq, h.max_dep, sol, sp->phys.phi.p, sp->dev.t_n.p,
                                                         sp->dev.t_ind.p, sp->dev.t_val.p, out);
    TSEM_LAUNCHED();
}

void eval_qp(tsem_space_s* sp, const double* sol_host, double* out_host) {
    physics_basis(sp);
    auto& h = sp->host;
    cudaStream_t s = sp->stream;
    const int nq = (int)sp->quad.w3.size();
    DBuf<double> sol, out((size_t)h.nt * nq);
    sol.upload(sol_host, h.n_dof, s);
    eval_qp_device(sp, sol.p, out.p, s);
    out.download(out_host, (size_t)h.nt * nq, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
}

// occupation numbers of up to kDensityMax states, passed by value
constexpr int kDensityMax = 64;
struct Occupations {
    double v[kDensityMax];
};

// Occupation-weighted density of k states at the element quadrature points,
// rho(x_q) = sum_j occ_j psi_j(x_q)^2 (calc_density, src/PointInfo.cpp:72-91); state j
// at u + j n.  With v set, the density difference d = sum_j occ_j (u_j^2 - v_j^2) is
// integrated instead (calc_density_l2_difference, src/CalcError.cpp:703-735):
// out[e] = |T_e| sum_q w_q d_q^2.  One block per element; the coefficients of one
// state sit in shared memory, the sum over states in acc [E][nq] (global: a rule may
// have tens of thousands of points), each point owned by one thread throughout.
__global__ void k_density(int n_loc, int nq, int max_dep, int k, int64_t n, const double* __restrict__ u,
                          const double* __restrict__ v, Occupations occ, const double* __restrict__ phi,
                          const int* __restrict__ t_n, const int* __restrict__ t_ind, const double* __restrict__ t_val,
                          const double* __restrict__ w, const double* __restrict__ vol, double* __restrict__ acc,
                          double* __restrict__ out) {
    const int e = blockIdx.x;
    extern __shared__ double sm[];
    double* cu = sm;
    double* cv = sm + n_loc;
    double* d = acc + (size_t)e * nq;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) d[q] = 0;
    for (int j = 0; j < k; ++j) {
        __syncthreads();   // the previous state's coefficients are used up
        for (int i = threadIdx.x; i < n_loc; i += blockDim.x) {
            const size_t b = (size_t)e * n_loc + i;
            double su = 0, sv = 0;
            for (int m = 0; m < t_n[b]; ++m) {
                const int64_t g = (int64_t)j * n + t_ind[b * max_dep + m];
                const double tv = t_val[b * max_dep + m];
                su += u[g] * tv;
                if (v) sv += v[g] * tv;
            }
            cu[i] = su;
            cv[i] = sv;
        }
        __syncthreads();
        const double o = occ.v[j];
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            double a = 0, c = 0;
            for (int i = 0; i < n_loc; ++i) {
                const double ph = phi[(size_t)q * n_loc + i];
                a += cu[i] * ph;
                if (v) c += cv[i] * ph;
            }
            // each square rounded on its own (no contraction), as the reference's
            // pow(u, 2) - pow(v, 2): equal states give exactly zero
            d[q] += o * (__dmul_rn(a, a) - __dmul_rn(c, c));   // each q stays with one thread
        }
    }
    if (!v) return;   // the density is acc itself
    double sq = 0;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) sq += w[q] * d[q] * d[q];
    for (int off = 16; off > 0; off >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, off);
    __shared__ double part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += part[i];
        out[e] = s * vol[e];
    }
}

static Occupations occupations(int k, const double* occ) {
    if (k < 1 || k > kDensityMax) throw Error(TSEM_INVALID, "the number of states must be 1.." + std::to_string(kDensityMax));
    Occupations o{};
    for (int j = 0; j < k; ++j) o.v[j] = occ[j];
    return o;
}

// acc: [E][nq] (the density itself when v is null), out: [E] partial integrals otherwise
static void launch_density(tsem_space_s* sp, int k, const double* u, const double* v, const Occupations& o,
                           double* acc, double* out, cudaStream_t s) {
    auto& h = sp->host;
    const int nq = (int)sp->quad.w3.size();
    const size_t smem = 2 * (size_t)h.n_loc * sizeof(double);
    k_density<<<h.nt, 128, smem, s>>>(h.n_loc, nq, h.max_dep, k, h.n_dof, u, v, o, sp->phys.phi.p, sp->dev.t_n.p,
                                      sp->dev.t_ind.p, sp->dev.t_val.p, sp->dev.w3.p, sp->dev.volume.p, acc, out);
    TSEM_LAUNCHED();
}

// device arrays, enqueued on s: states [k][n_dof], out [E][nq]
void density_device(tsem_space_s* sp, const double* states, int k, const double* occ, double* out, cudaStream_t s) {
    const Occupations o = occupations(k, occ);
    physics_basis(sp);
    TSEM_CUDA(cudaStreamSynchronize(sp->stream));   // the space's device data is in place
    launch_density(sp, k, states, nullptr, o, out, nullptr, s);
}

void density(tsem_space_s* sp, const double* states_host, int k, const double* occ, double* out_host) {
    const Occupations o = occupations(k, occ);
    physics_basis(sp);
    auto& h = sp->host;
    cudaStream_t s = sp->stream;
    const int nq = (int)sp->quad.w3.size();
    DBuf<double> st, out((size_t)h.nt * nq);
    st.upload(states_host, (size_t)k * h.n_dof, s);
    launch_density(sp, k, st.p, nullptr, o, out.p, nullptr, s);
    out.download(out_host, (size_t)h.nt * nq, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
}

double density_l2_difference(tsem_space_s* sp, const double* u_host, const double* v_host, int k, const double* occ) {
    const Occupations o = occupations(k, occ);
    physics_basis(sp);
    auto& h = sp->host;
    cudaStream_t s = sp->stream;
    DBuf<double> u, v, part(h.nt), d((size_t)h.nt * sp->quad.w3.size());
    u.upload(u_host, (size_t)k * h.n_dof, s);
    v.upload(v_host, (size_t)k * h.n_dof, s);
    launch_density(sp, k, u.p, v.p, o, d.p, part.p, s);
    std::vector<double> hp(h.nt);
    part.download(hp.data(), h.nt, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    double sum = 0;
    for (double x : hp) sum += x;   // element order: the result does not depend on the launch
    return std::sqrt(sum);
}

// dst += alpha src entry by entry (src's pattern inside dst's); one thread per row of src
__global__ void k_csr_axpy(int64_t n, const int64_t* __restrict__ rps, const int* __restrict__ cs,
                           const double* __restrict__ vs, double alpha, const int64_t* __restrict__ rpd,
                           const int* __restrict__ cd, double* vd, int* err) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        for (int64_t k = rps[r]; k < rps[r + 1]; ++k) {
            const int64_t p = find_col(rpd, cd, (int)r, cs[k]);
            if (p < 0) { atomicExch(err, 1); continue; }
            vd[p] += alpha * vs[k];
        }
}

void csr_axpy(DevCsr& dst, double alpha, const DevCsr& src, cudaStream_t s) {
    if (dst.n != src.n) throw Error(TSEM_INVALID, "matrix sizes differ");
    DBuf<int> err(1);
    err.zero(s);
    k_csr_axpy<<<grid_for(src.n, 256), 256, 0, s>>>(src.n, src.rowptr.p, src.col.p, src.val.p, alpha, dst.rowptr.p,
                                                    dst.col.p, dst.val.p, err.p);
    TSEM_LAUNCHED();
    dst.refresh_diag(s);
    dst.spmv_variant = -1;
    int herr = 0;
    err.download(&herr, 1, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    if (herr) throw Error(TSEM_INVALID, "the added matrix has entries outside the pattern of the target");
}

}  // namespace tsem

namespace tsem {

// ----------------------------------------------------------- interpolation
// calc_interpolation (src/Interpolation.cpp:104-216), interior part: per element the
// non-interior local coefficients are recovered through T_e, subtracted from f at the
// quadrature points, and every interior mode (l1-2, l2-1, l3-1) is the weighted
// integral against its collapsed Jacobi product (scale folded into interp3).
__global__ void k_interp_interior(int n_loc, int nq, int max_dep, const double* __restrict__ f,
                                  const double* __restrict__ w, const double* __restrict__ phi,
                                  const double* __restrict__ interp3, const uint8_t* __restrict__ interior,
                                  const int* __restrict__ t_n, const int* __restrict__ t_ind,
                                  const double* __restrict__ t_val, double* fr_all, double* val) {
    const int e = blockIdx.x;
    extern __shared__ double shm[];
    double* c = shm;                          // [n_loc]
    double* fr = fr_all + (size_t)e * nq;     // [nq], global: a rule may have tens of thousands of points
    for (int i = threadIdx.x; i < n_loc; i += blockDim.x) {
        double v = 0.0;
        if (!interior[i]) {
            const size_t b = (size_t)e * n_loc + i;
            for (int j = 0; j < t_n[b]; ++j) v += val[t_ind[b * max_dep + j]] * t_val[b * max_dep + j];
        }
        c[i] = v;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        double v = f[(size_t)e * nq + q];
        for (int i = 0; i < n_loc; ++i) v -= c[i] * phi[(size_t)q * n_loc + i];
        fr[q] = w[q] * v;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_loc; i += blockDim.x) {
        if (!interior[i]) continue;
        double v = 0.0;
        for (int q = 0; q < nq; ++q) v += fr[q] * interp3[(size_t)q * n_loc + i];
        const size_t b = (size_t)e * n_loc + i;
        val[t_ind[b * max_dep]] = v;   // interior modes: one term, coefficient 1
    }
}

void interpolation(tsem_space_s* sp, const double* uv, const double* ue, const double* uf, const double* u_qp,
                   double* out_host) {
    physics_faces(sp);
    physics_basis(sp);
    auto& h = sp->host;
    auto& F = sp->phys;
    cudaStream_t s = sp->stream;
    const int nq = (int)sp->quad.w3.size(), nl = h.n_loc, M = h.M;
    // interior table, host: interp3[q][a] = scale(a) * product of the collapsed Jacobi factors
    std::vector<double> it((size_t)nq * nl, 0.0);
    std::vector<uint8_t> inter(nl, 0);
    std::vector<double> P1(M + 2), P2(M + 2), P3(M + 2);
    for (int a = 0; a < nl; ++a) {
        const auto al = mi_index(a);
        inter[a] = al[0] >= 2 && al[1] >= 1 && al[2] >= 1;
    }
    for (int q = 0; q < nq; ++q) {
        const double x = sp->quad.x3[3 * q], y = sp->quad.x3[3 * q + 1], z = sp->quad.x3[3 * q + 2];
        const double xi = 2 * x / (1 - y - z) - 1, eta = 2 * y / (1 - z) - 1, zeta = 2 * z - 1;
        jacobi_classic<double>(1, 1, xi, std::max(M - 2, 0), P1.data());
        for (int a = 0; a < nl; ++a) {
            if (!inter[a]) continue;
            const auto al = mi_index(a);
            const int l1 = al[0], l2 = al[1], l3 = al[2];
            jacobi_classic<double>(2 * l1 - 1, 1, eta, std::max(l2 - 1, 0), P2.data());
            jacobi_classic<double>(2 * l1 + 2 * l2 - 1, 1, zeta, std::max(l3 - 1, 0), P3.data());
            const double B = P1[l1 - 2] * std::pow(1 - eta, l1 - 2) * P2[l2 - 1] * std::pow(1 - zeta, l1 + l2 - 3) *
                             P3[l3 - 1];
            const double scale = -(double)l1 * (2 * l1 - 1) * (2 * l1 + 2 * l2 - 1) * (2 * l1 + 2 * l2 + 2 * l3 - 1) /
                                 (std::pow(2.0, 2 * l1 + l2 - 5) * (l1 - 1) * 6.0);
            it[(size_t)q * nl + a] = scale * B;
        }
    }
    DBuf<double> du_v, du_e, du_f, dq, val(h.n_dof), t3;
    DBuf<uint8_t> isd(h.n_dof), din;
    du_v.upload(uv, h.nv, s);
    du_e.upload(ue, (size_t)h.ne * F.fb.nq1, s);
    du_f.upload(uf, (size_t)h.nf * F.fb.nq2, s);
    dq.upload(u_qp, (size_t)h.nt * nq, s);
    t3.upload(it, s);
    din.upload(inter, s);
    val.zero(s);
    isd.zero(s);
    k_dir_vertex<<<grid_for(h.nv, 256), 256, 0, s>>>(h.nv, -2, F.mark_v.p, du_v.p, F.vdof.p, val.p, isd.p);
    TSEM_LAUNCHED();
    if (h.ndE > 0) {
        k_dir_edge<<<grid_for((int64_t)h.ne * h.ndE, 256), 256, 0, s>>>(h.ne, F.fb.nq1, h.ndE, -2, F.mark_e.p, du_e.p,
                                                                       F.edge_node.p, F.vdof.p, F.edof.p, F.x1.p, F.w1.p,
                                                                       F.interp1.p, val.p, isd.p);
        TSEM_LAUNCHED();
    }
    if (h.ndF > 0) {
        k_dir_face<<<grid_for((int64_t)h.nf * h.ndF, 128), 128, 0, s>>>(h.nf, F.fb.nq2, h.ndE, h.ndF, h.M, -2, F.mark_f.p,
                                                                       du_f.p, F.face_node.p, F.face_edge.p, F.face_same.p,
                                                                       F.vdof.p, F.edof.p, F.fdof.p, F.b2.p, F.w2.p, F.add0.p,
                                                                       F.add1.p, F.interp2.p, val.p, isd.p);
        TSEM_LAUNCHED();
    }
    DBuf<double> fr((size_t)h.nt * nq);
    k_interp_interior<<<h.nt, 128, (size_t)nl * sizeof(double), s>>>(nl, nq, h.max_dep, dq.p, sp->dev.w3.p,
                                                                     F.phi.p, t3.p, din.p, sp->dev.t_n.p,
                                                                     sp->dev.t_ind.p, sp->dev.t_val.p, fr.p, val.p);
    TSEM_LAUNCHED();
    val.download(out_host, h.n_dof, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
}

}  // namespace tsem
