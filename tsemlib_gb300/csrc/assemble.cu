// Reference-element matrices by exact quadrature and global CSR assembly on the GPU.
//
// Assembly follows TSEMLib's build_stiff_matrix / build_mass_matrix
// (src/Discretize.cpp:1297-1395, :522-665): the global pattern is the diagonal plus,
// for every element and every structural entry (a, c) of the reference matrices,
// all pairs (dep(a), dep(c)) of the global->local transform; values are scattered
// as  v(a,c) * t_a * t_c  with v = (2 / (3|T|)) sum_k G_k S_k(a,c)  (stiffness) or
// 6|T| M(a,c)  (mass).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <numeric>

#include "device.hpp"
#include "jacobi.cuh"

namespace tsem {

void ensure_stream(cudaStream_t* s, int* device) {
    if (*s) return;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        throw Error(TSEM_NO_DEVICE, "no CUDA device available");
    }
    TSEM_CUDA(cudaGetDevice(device));
    TSEM_CUDA(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking));
}

void space_upload(tsem_space_s* sp) {
    if (sp->dev.ready) return;
    ensure_stream(&sp->stream, &sp->device);
    auto& h = sp->host;
    auto& d = sp->dev;
    cudaStream_t s = sp->stream;
    d.t_n.upload(h.t_n, s);
    d.t_ind.upload(h.t_ind, s);
    d.t_val.upload(h.t_val, s);
    d.xyz.upload(h.xyz, s);
    d.volume.upload(h.volume, s);
    d.ele_node.upload(h.ele_node, s);
    d.x3.upload(sp->quad.x3, s);
    d.w3.upload(sp->quad.w3, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    d.ready = true;
}

// ------------------------------------------------------------ reference matrices
constexpr int kMaxOrder = 16;

// phi and grad phi (actual basis) at quadrature point q; out_v [nq][n], out_g [nq][n][3]
__global__ void k_basis_at_points(int M, int n, int nq, const double* __restrict__ pts, const int* __restrict__ ts,
                                  const int* __restrict__ tt, const double* __restrict__ tw, double* out_v,
                                  double* out_g, Dual* scratch) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    Dual* J = scratch + (size_t)q * n;
    const Dual x(pts[3 * q], 1, 0, 0), y(pts[3 * q + 1], 0, 1, 0), z(pts[3 * q + 2], 0, 0, 1);
    jacobi_products<Dual, kMaxOrder>(M, x, y, z, J);
    double* v = out_v + (size_t)q * n;
    double* g = out_g + (size_t)q * n * 3;
    for (int i = 0; i < n; ++i) { v[i] = 0; g[3 * i] = 0; g[3 * i + 1] = 0; g[3 * i + 2] = 0; }
    for (int a = 0; a < n; ++a)
        for (int j = ts[a]; j < ts[a + 1]; ++j) {
            const int t = tt[j];
            const double w = tw[j];
            v[t] += w * J[a].v;
            g[3 * t] += w * J[a].d0;
            g[3 * t + 1] += w * J[a].d1;
            g[3 * t + 2] += w * J[a].d2;
        }
}

// M(i,j) = sum_q w_q phi_i phi_j / 6 ;  S_k(i,j) = sum_q w_q (d_k . grad phi_i)(d_k . grad phi_j) / 6
__global__ void k_reference_gram(int n, int nq, const double* __restrict__ w, const double* __restrict__ v,
                                 const double* __restrict__ g, double* mass, double* stiff) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * n) return;
    const int i = idx / n, j = idx % n;
    // directions of the six edge derivatives: x1, x2-x1, x1-x3, x2, x3-x2, x3
    const double D[6][3] = {{1, 0, 0}, {-1, 1, 0}, {1, 0, -1}, {0, 1, 0}, {0, -1, 1}, {0, 0, 1}};
    double m = 0, s[6] = {0, 0, 0, 0, 0, 0};
    for (int q = 0; q < nq; ++q) {
        const double wq = w[q];
        m += wq * v[(size_t)q * n + i] * v[(size_t)q * n + j];
        const double* gi = g + ((size_t)q * n + i) * 3;
        const double* gj = g + ((size_t)q * n + j) * 3;
        for (int k = 0; k < 6; ++k) {
            const double a = D[k][0] * gi[0] + D[k][1] * gi[1] + D[k][2] * gi[2];
            const double b = D[k][0] * gj[0] + D[k][1] * gj[1] + D[k][2] * gj[2];
            s[k] += wq * a * b;
        }
    }
    mass[idx] = m / 6.0;
    for (int k = 0; k < 6; ++k) stiff[(size_t)k * n * n + idx] = s[k] / 6.0;
}

void space_reference(tsem_space_s* sp) {
    if (sp->ref) return;
    space_upload(sp);
    cudaStream_t s = sp->stream;
    auto& h = sp->host;
    const int M = h.M, n = h.n_loc;
    // exact for the degree-2M integrands in collapsed coordinates
    Quadrature Q;
    Q.build(M + 3);
    const int nq = (int)Q.w3.size();
    DBuf<double> pts, w, v, g, mass, stiff;
    DBuf<int> ts, tt;
    DBuf<double> tw;
    DBuf<Dual> scratch((size_t)nq * n);
    pts.upload(Q.x3, s);
    w.upload(Q.w3, s);
    ts.upload(h.lt.start, s);
    tt.upload(h.lt.target, s);
    tw.upload(h.lt.weight, s);
    v.alloc((size_t)nq * n);
    g.alloc((size_t)nq * n * 3);
    mass.alloc((size_t)n * n);
    stiff.alloc((size_t)6 * n * n);
    k_basis_at_points<<<(nq + 63) / 64, 64, 0, s>>>(M, n, nq, pts.p, ts.p, tt.p, tw.p, v.p, g.p, scratch.p);
    TSEM_LAUNCHED();
    k_reference_gram<<<(n * n + 127) / 128, 128, 0, s>>>(n, nq, w.p, v.p, g.p, mass.p, stiff.p);
    TSEM_LAUNCHED();
    auto R = std::make_unique<ReferenceMatrices>();
    R->n_loc = n;
    R->mass.resize((size_t)n * n);
    R->stiff.resize((size_t)6 * n * n);
    mass.download(R->mass.data(), R->mass.size(), s);
    stiff.download(R->stiff.data(), R->stiff.size(), s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    // keep the reference's structural patterns only
    for (size_t i = 0; i < (size_t)n * n; ++i) {
        if (!h.pat.mass[i]) R->mass[i] = 0.0;
        for (int k = 0; k < 6; ++k)
            if (!h.pat.stiff[k][i]) R->stiff[(size_t)k * n * n + i] = 0.0;
    }
    std::vector<int> mp, spairs;
    std::vector<double> mv, sv;
    for (int i = 0; i < n * n; ++i) {
        if (h.pat.mass[i]) { mp.push_back(i); mv.push_back(R->mass[i]); }
        if (h.pat.stiff_union[i]) {
            spairs.push_back(i);
            for (int k = 0; k < 6; ++k) sv.push_back(R->stiff[(size_t)k * n * n + i]);
        }
    }
    R->n_mass_pairs = (int64_t)mp.size();
    R->n_stiff_pairs = (int64_t)spairs.size();
    R->mass_pairs.upload(mp, s);
    R->mass_vals.upload(mv, s);
    R->stiff_pairs.upload(spairs, s);
    R->stiff_vals.upload(sv, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    sp->ref = std::move(R);
}

// --------------------------------------------------------------------- assembly
__device__ __forceinline__ int64_t lower_bound_i32(const int* __restrict__ a, int64_t lo, int64_t hi, int key) {
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// mark the structural (row, col) pairs inside the candidate lists; one block per element
__global__ void k_mark_pattern(int n_loc, int max_dep, int64_t n_pairs, const int* __restrict__ pairs,
                               const int* __restrict__ t_n, const int* __restrict__ t_ind,
                               const int* __restrict__ row_geo, const int64_t* __restrict__ geo_start,
                               const int* __restrict__ cand, const int64_t* __restrict__ flag_off, uint8_t* flags,
                               int* err) {
    const int e = blockIdx.x;
    for (int64_t pi = threadIdx.x; pi < n_pairs; pi += blockDim.x) {
        const int a = pairs[pi] / n_loc, c = pairs[pi] % n_loc;
        const size_t ba = (size_t)e * n_loc + a, bc = (size_t)e * n_loc + c;
        const int na = t_n[ba], nc = t_n[bc];
        for (int u = 0; u < na; ++u) {
            const int row = t_ind[ba * max_dep + u];
            const int gl = row_geo[row];
            const int64_t lo = geo_start[gl], hi = geo_start[gl + 1];
            for (int w = 0; w < nc; ++w) {
                const int colv = t_ind[bc * max_dep + w];
                const int64_t pos = lower_bound_i32(cand, lo, hi, colv);
                if (pos >= hi || cand[pos] != colv) { atomicExch(err, 1); continue; }
                flags[flag_off[row] + (pos - lo)] = 1;
            }
        }
    }
}

__global__ void k_count_rows(int64_t n, const int* __restrict__ row_geo, const int64_t* __restrict__ geo_start,
                             const int* __restrict__ cand, const int64_t* __restrict__ flag_off,
                             const uint8_t* __restrict__ flags, int64_t* counts) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const int gl = row_geo[r];
        const int64_t len = geo_start[gl + 1] - geo_start[gl];
        int64_t c = 0;
        bool diag = false;
        for (int64_t k = 0; k < len; ++k)
            if (flags[flag_off[r] + k]) {
                ++c;
                if (cand[geo_start[gl] + k] == (int)r) diag = true;
            }
        counts[r] = c + (diag ? 0 : 1);
    }
}

__global__ void k_fill_rows(int64_t n, const int* __restrict__ row_geo, const int64_t* __restrict__ geo_start,
                            const int* __restrict__ cand, const int64_t* __restrict__ flag_off,
                            const uint8_t* __restrict__ flags, const int64_t* __restrict__ rowptr, int* col) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const int gl = row_geo[r];
        const int64_t len = geo_start[gl + 1] - geo_start[gl];
        int64_t o = rowptr[r];
        col[o++] = (int)r;                   // diagonal first (deal.II square convention)
        for (int64_t k = 0; k < len; ++k) {
            const int cv = cand[geo_start[gl] + k];
            if (flags[flag_off[r] + k] && cv != (int)r) col[o++] = cv;
        }
    }
}

// G_k of src/Discretize.cpp:1357-1372 for the six face pairs of a tetrahedron
__device__ void dihedral_weights(const double* __restrict__ xyz, const int* nodes, double g[6]) {
    double P[4][3];
    for (int k = 0; k < 4; ++k)
        for (int j = 0; j < 3; ++j) P[k][j] = xyz[3 * (size_t)nodes[k] + j];
    // face pair (i1, i2) -> common edge (s, t) and matrix slot
    const int I1[6] = {0, 0, 0, 1, 1, 2}, I2[6] = {1, 2, 3, 2, 3, 3};
    const int Sx[6] = {2, 1, 2, 0, 0, 0}, Tx[6] = {3, 3, 1, 3, 2, 1};
    const int slot[6] = {0, 3, 5, 1, 2, 4};
    for (int q = 0; q < 6; ++q) {
        double a[3], b[3], c[3];
        for (int j = 0; j < 3; ++j) {
            a[j] = P[Tx[q]][j] - P[Sx[q]][j];
            b[j] = P[I1[q]][j] - P[Sx[q]][j];
            c[j] = P[I2[q]][j] - P[Sx[q]][j];
        }
        const double u0 = a[1] * b[2] - a[2] * b[1], u1 = -a[0] * b[2] + a[2] * b[0], u2 = a[0] * b[1] - a[1] * b[0];
        const double v0 = a[1] * c[2] - a[2] * c[1], v1 = -a[0] * c[2] + a[2] * c[0], v2 = a[0] * c[1] - a[1] * c[0];
        const double w = 0.25 * (u0 * v0 + u1 * v1 + u2 * v2);
        g[slot[q]] = fabs(w) < 1e-12 ? 0.0 : w;
    }
}

__device__ __forceinline__ int64_t csr_find(const int64_t* __restrict__ rowptr, const int* __restrict__ col, int r, int c) {
    const int64_t b = rowptr[r], e = rowptr[r + 1];
    if (col[b] == c) return b;
    const int64_t p = lower_bound_i32(col, b + 1, e, c);
    return (p < e && col[p] == c) ? p : -1;
}

// one block per element; threads stride over the structural pairs
__global__ void k_scatter(int which, int n_loc, int max_dep, int64_t n_pairs, const int* __restrict__ pairs,
                          const double* __restrict__ pvals, const int* __restrict__ t_n, const int* __restrict__ t_ind,
                          const double* __restrict__ t_val, const double* __restrict__ xyz,
                          const int* __restrict__ ele_node, const double* __restrict__ volume,
                          const int64_t* __restrict__ rowptr, const int* __restrict__ col, double* val, int* err) {
    const int e = blockIdx.x;
    __shared__ double g[6];
    __shared__ double coef;
    if (threadIdx.x == 0) {
        if (which == 0) {
            dihedral_weights(xyz, ele_node + 4 * (size_t)e, g);
            coef = 2.0 / (3.0 * volume[e]);
        } else {
            coef = 6.0 * volume[e];
        }
    }
    __syncthreads();
    for (int64_t pi = threadIdx.x; pi < n_pairs; pi += blockDim.x) {
        double v;
        if (which == 0) {
            const double* s = pvals + pi * 6;
            v = coef * (g[0] * s[0] + g[1] * s[1] + g[2] * s[2] + g[3] * s[3] + g[4] * s[4] + g[5] * s[5]);
        } else {
            v = coef * pvals[pi];
        }
        if (v == 0.0) continue;
        const int a = pairs[pi] / n_loc, c = pairs[pi] % n_loc;
        const size_t ba = (size_t)e * n_loc + a, bc = (size_t)e * n_loc + c;
        const int na = t_n[ba], nc = t_n[bc];
        for (int u = 0; u < na; ++u) {
            const int r = t_ind[ba * max_dep + u];
            const double vr = v * t_val[ba * max_dep + u];
            for (int w = 0; w < nc; ++w) {
                const int64_t p = csr_find(rowptr, col, r, t_ind[bc * max_dep + w]);
                if (p < 0) { atomicExch(err, 1); continue; }
                atomicAdd(val + p, vr * t_val[bc * max_dep + w]);
            }
        }
    }
}

__global__ void k_extract_diag(int64_t n, const int64_t* __restrict__ rowptr, const double* __restrict__ val, double* d) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        d[r] = val[rowptr[r]];
}

void DevCsr::refresh_diag(cudaStream_t s) {
    values_changed();
    if (diag.n != (size_t)n) diag.alloc(n);
    k_extract_diag<<<grid_for(n, 256), 256, 0, s>>>(n, rowptr.p, val.p, diag.p);
    TSEM_LAUNCHED();
}

// CSR pattern of the element pairs (a, c) in `pairs` through every element's
// transform: rows diagonal first, then ascending columns
static void build_pattern(tsem_space_s* sp, const int* pairs, int64_t np, DevCsr& out) {
    cudaStream_t s = sp->stream;
    auto& h = sp->host;
    auto& d = sp->dev;
    if (!sp->cand) {
        sp->cand = std::make_unique<PatternCandidates>();
        sp->cand->build(h);
    }
    const PatternCandidates& C = *sp->cand;
    const int64_t n = h.n_dof;
    std::vector<int64_t> flag_off(n + 1, 0);
    for (int64_t r = 0; r < n; ++r) {
        const int gl = C.row_geo[r];
        flag_off[r + 1] = flag_off[r] + (C.geo_start[gl + 1] - C.geo_start[gl]);
    }
    DBuf<int> row_geo, cand;
    DBuf<int64_t> geo_start, off, counts;
    DBuf<uint8_t> flags(flag_off[n]);
    row_geo.upload(C.row_geo, s);
    cand.upload(C.cand, s);
    geo_start.upload(C.geo_start, s);
    off.upload(flag_off, s);
    flags.zero(s);
    DBuf<int> err(1);
    err.zero(s);
    k_mark_pattern<<<h.nt, 256, 0, s>>>(h.n_loc, h.max_dep, np, pairs, d.t_n.p, d.t_ind.p, row_geo.p, geo_start.p,
                                        cand.p, off.p, flags.p, err.p);
    TSEM_LAUNCHED();
    counts.alloc(n);
    k_count_rows<<<grid_for(n, 256), 256, 0, s>>>(n, row_geo.p, geo_start.p, cand.p, off.p, flags.p, counts.p);
    TSEM_LAUNCHED();
    std::vector<int64_t> rp(n + 1, 0);
    counts.download(rp.data() + 1, n, s);
    int herr = 0;
    err.download(&herr, 1, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    if (herr) throw Error(TSEM_INVALID, "a transform term falls outside the candidate lists");
    for (int64_t r = 0; r < n; ++r) rp[r + 1] += rp[r];
    out.n = n;
    out.nnz = rp[n];
    out.rowptr.upload(rp, s);
    out.col.alloc(out.nnz);
    out.val.alloc(out.nnz);
    out.val.zero(s);
    k_fill_rows<<<grid_for(n, 256), 256, 0, s>>>(n, row_geo.p, geo_start.p, cand.p, off.p, flags.p, out.rowptr.p, out.col.p);
    TSEM_LAUNCHED();
    TSEM_CUDA(cudaStreamSynchronize(s));
}

void space_pattern_full(tsem_space_s* sp, DevCsr& out) {
    space_upload(sp);
    const int nl = sp->host.n_loc;
    std::vector<int> all((size_t)nl * nl);
    for (int i = 0; i < nl * nl; ++i) all[i] = i;
    DBuf<int> pairs;
    pairs.upload(all, sp->stream);
    build_pattern(sp, pairs.p, (int64_t)all.size(), out);
}

void space_assemble(tsem_space_s* sp, int which, DevCsr& out) {
    space_reference(sp);
    cudaStream_t s = sp->stream;
    auto& h = sp->host;
    auto& d = sp->dev;
    auto& R = *sp->ref;
    const int* pairs = which == 0 ? R.stiff_pairs.p : R.mass_pairs.p;
    const int64_t np = which == 0 ? R.n_stiff_pairs : R.n_mass_pairs;
    const double* pvals = which == 0 ? R.stiff_vals.p : R.mass_vals.p;
    build_pattern(sp, pairs, np, out);
    DBuf<int> err(1);
    err.zero(s);
    k_scatter<<<h.nt, 256, 0, s>>>(which, h.n_loc, h.max_dep, np, pairs, pvals, d.t_n.p, d.t_ind.p, d.t_val.p, d.xyz.p,
                                   d.ele_node.p, d.volume.p, out.rowptr.p, out.col.p, out.val.p, err.p);
    TSEM_LAUNCHED();
    out.refresh_diag(s);
    int herr = 0;
    err.download(&herr, 1, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    if (herr) throw Error(TSEM_INVALID, "assembly met an entry outside the structural pattern");
}


}  // namespace tsem
