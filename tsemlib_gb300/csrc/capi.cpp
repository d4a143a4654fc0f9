// The C ABI (include/tsem_gpu.h): argument checks, exception -> status mapping.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <string>

#include "device.hpp"
#include "jacobi.cuh"
#include "lobpcg.hpp"
#include "solver.hpp"

using namespace tsem;

namespace {
thread_local std::string g_err;

tsem_status fail(tsem_status s, const std::string& m) {
    g_err = m;
    return s;
}

template <class F>
tsem_status guard(F&& f) {
    try {
        f();
        return TSEM_OK;
    } catch (const Error& e) {
        return fail(e.status, e.what());
    } catch (const std::invalid_argument& e) {
        return fail(TSEM_INVALID, e.what());
    } catch (const std::bad_alloc&) {
        return fail(TSEM_OOM_REFUSED, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(TSEM_INVALID, e.what());
    }
}

#define REQUIRE(cond, msg) \
    if (!(cond)) return fail(TSEM_INVALID, msg)

cudaStream_t pick(void* user, cudaStream_t own) { return user ? (cudaStream_t)user : own; }
}  // namespace

extern "C" {

const char* tsem_last_error(void) { return g_err.c_str(); }

int64_t tsem_kernel_launches(void) { return g_kernel_launches.load(); }

tsem_status tsem_space_create(const tsem_mesh* m, int32_t p, int32_t quad_q, tsem_space* out) {
    REQUIRE(m && out, "null argument");
    REQUIRE(quad_q >= 1 && quad_q <= 64, "quad_q must be in [1, 64]");
    *out = nullptr;
    return guard([&] {
        auto sp = std::make_unique<tsem_space_s>();
        MeshInput in;
        in.nv = m->nv; in.ne = m->ne; in.nf = m->nf; in.nt = m->nt;
        in.xyz = m->xyz; in.edge_v = m->edge_v; in.face_v = m->face_v; in.face_e = m->face_e;
        in.tet_v = m->tet_v; in.tet_f = m->tet_f;
        in.mark_v = m->mark_v; in.mark_e = m->mark_e; in.mark_f = m->mark_f;
        in.femdof_v = m->femdof_v; in.femdof_e = m->femdof_e;
        sp->host.build(in, p);
        sp->quad.build(quad_q);
        *out = sp.release();
    });
}

tsem_status tsem_space_set_quadrature(tsem_space s, int32_t n1, const double* x1, const double* w1, int32_t n2,
                                      const double* b2, const double* w2, int32_t n3, const double* x3,
                                      const double* w3) {
    REQUIRE(s && x1 && w1 && b2 && w2 && x3 && w3, "null argument");
    REQUIRE(n1 > 0 && n2 > 0 && n3 > 0, "every rule needs at least one point");
    return guard([&] {
        Quadrature Q;
        Q.q = 0;
        Q.x1.assign(x1, x1 + n1);
        Q.w1.assign(w1, w1 + n1);
        Q.b2.assign(b2, b2 + 3 * (size_t)n2);
        Q.w2.assign(w2, w2 + n2);
        Q.x3.assign(x3, x3 + 3 * (size_t)n3);
        Q.w3.assign(w3, w3 + n3);
        if (s->stream) TSEM_CUDA(cudaStreamSynchronize(s->stream));
        s->quad = std::move(Q);
        // device copies of the rule and of the bases at its points are rebuilt on demand
        s->dev.ready = false;
        s->phys.ready = false;
        s->phys.faces_ready = false;
        s->phys.pair2.release();
    });
}

void tsem_space_destroy(tsem_space s) {
    if (!s) return;
    cudaStream_t st = s->stream;
    delete s;
    if (st) cudaStreamDestroy(st);
    trace_mark("space_destroy");
}

tsem_status tsem_space_info(tsem_space s, int64_t* info) {
    REQUIRE(s && info, "null argument");
    auto& h = s->host;
    info[0] = h.n_dof; info[1] = h.n_loc; info[2] = h.nt; info[3] = h.max_dep;
    info[4] = (int64_t)s->quad.w3.size(); info[5] = (int64_t)s->quad.w2.size(); info[6] = (int64_t)s->quad.w1.size();
    info[7] = h.nv; info[8] = h.ne; info[9] = h.nf; info[10] = h.nt;
    info[11] = 1; info[12] = h.ndE; info[13] = h.ndF; info[14] = h.ndI;
    return TSEM_OK;
}

tsem_status tsem_space_numbering(tsem_space s, int32_t* lg, int32_t* la) {
    REQUIRE(s, "null argument");
    if (lg) std::copy(s->host.location_geometry.begin(), s->host.location_geometry.end(), lg);
    if (la) std::copy(s->host.location_actualdof.begin(), s->host.location_actualdof.end(), la);
    return TSEM_OK;
}

tsem_status tsem_space_transform(tsem_space s, int32_t* t_n, int32_t* t_ind, double* t_val) {
    REQUIRE(s, "null argument");
    auto& h = s->host;
    if (t_n) std::copy(h.t_n.begin(), h.t_n.end(), t_n);
    if (t_ind) std::copy(h.t_ind.begin(), h.t_ind.end(), t_ind);
    if (t_val) std::copy(h.t_val.begin(), h.t_val.end(), t_val);
    return TSEM_OK;
}

tsem_status tsem_space_geometry(tsem_space s, int8_t* type_edge, int8_t* type_face, int8_t* type_face_inv,
                                int32_t* edge_node, int32_t* face_node, int32_t* face_edge, uint8_t* face_same,
                                double* volume) {
    REQUIRE(s, "null argument");
    auto& h = s->host;
    if (type_edge) std::copy(h.type_edge.begin(), h.type_edge.end(), type_edge);
    if (type_face) std::copy(h.type_face.begin(), h.type_face.end(), type_face);
    if (type_face_inv) std::copy(h.type_face_inv.begin(), h.type_face_inv.end(), type_face_inv);
    if (edge_node) std::copy(h.edge_node.begin(), h.edge_node.end(), edge_node);
    if (face_node) std::copy(h.face_node.begin(), h.face_node.end(), face_node);
    if (face_edge) std::copy(h.face_edge.begin(), h.face_edge.end(), face_edge);
    if (face_same) std::copy(h.face_same.begin(), h.face_same.end(), face_same);
    if (volume) std::copy(h.volume.begin(), h.volume.end(), volume);
    return TSEM_OK;
}

tsem_status tsem_space_sum_dof(tsem_space s, int32_t* sum_dof) {
    REQUIRE(s && sum_dof, "null argument");
    std::copy(s->host.sum_dof.begin(), s->host.sum_dof.end(), sum_dof);
    return TSEM_OK;
}

tsem_status tsem_space_quadrature(tsem_space s, double* x3, double* w3, double* b2, double* w2, double* x1, double* w1) {
    REQUIRE(s, "null argument");
    auto& Q = s->quad;
    if (x3) std::copy(Q.x3.begin(), Q.x3.end(), x3);
    if (w3) std::copy(Q.w3.begin(), Q.w3.end(), w3);
    if (b2) std::copy(Q.b2.begin(), Q.b2.end(), b2);
    if (w2) std::copy(Q.w2.begin(), Q.w2.end(), w2);
    if (x1) std::copy(Q.x1.begin(), Q.x1.end(), x1);
    if (w1) std::copy(Q.w1.begin(), Q.w1.end(), w1);
    return TSEM_OK;
}

tsem_status tsem_element_qpoints(tsem_space s, double* out) {
    REQUIRE(s && out, "null argument");
    return guard([&] { element_qpoints(s, out); });
}

tsem_status tsem_boundary_points(tsem_space s, int32_t dim, double* out, int64_t* count) {
    REQUIRE(s && count, "null argument");
    REQUIRE(dim >= 0 && dim <= 2, "dim must be 0, 1 or 2");
    return guard([&] { boundary_points(s, dim, out, count); });
}

tsem_status tsem_geometry_marks(tsem_space s, int32_t dim, int32_t* out, int64_t* count) {
    REQUIRE(s && count, "null argument");
    REQUIRE(dim >= 0 && dim <= 2, "dim must be 0, 1 or 2");
    return guard([&] {
        const auto& h = s->host;
        const std::vector<int>& m = dim == 0 ? h.mark_v : dim == 1 ? h.mark_e : h.mark_f;
        *count = (int64_t)m.size();
        if (out) std::copy(m.begin(), m.end(), out);
    });
}

tsem_status tsem_multiindex(int32_t M, int32_t* alpha, int32_t* number) {
    REQUIRE(M >= 0 && M <= 40, "order must be in [0, 40]");
    const int n = mi_count(M);
    for (int i = 0; i < n; ++i) {
        const auto a = mi_index(i);
        if (alpha) std::copy(a.begin(), a.end(), alpha + 3 * (size_t)i);
        if (number) number[i] = mi_number(a[0], a[1], a[2]);
    }
    return TSEM_OK;
}

tsem_status tsem_face_table(int32_t p, int64_t* n_entries, int32_t* var, int32_t* dof, int32_t* kind, int32_t* edge_k,
                            int32_t* index, double* value) {
    REQUIRE(n_entries, "null argument");
    REQUIRE(p >= 1 && p <= 16, "order must be in [1, 16]");
    return guard([&] {
        FaceTable ft;
        ft.derive(p);
        int64_t c = 0;
        for (int v = 0; v < 6; ++v)
            for (int d = 0; d < ft.nf; ++d) {
                for (auto& t : ft.edge[v][d]) {
                    if (var) { var[c] = v; dof[c] = d; kind[c] = 0; edge_k[c] = t.k; index[c] = t.idx; value[c] = t.v; }
                    ++c;
                }
                for (auto& t : ft.face[v][d]) {
                    if (var) { var[c] = v; dof[c] = d; kind[c] = 1; edge_k[c] = -1; index[c] = t.idx; value[c] = t.v; }
                    ++c;
                }
            }
        *n_entries = c;
    });
}

tsem_status tsem_reference_matrix(tsem_space s, int32_t which, double* dense, uint8_t* pattern) {
    REQUIRE(s, "null argument");
    REQUIRE(which >= 0 && which <= 6, "which must be in [0, 6]");
    const int n = s->host.n_loc;
    if (pattern) {
        const auto& P = which == 0 ? s->host.pat.mass : s->host.pat.stiff[which - 1];
        std::copy(P.begin(), P.end(), pattern);
    }
    if (!dense) return TSEM_OK;
    return guard([&] {
        space_reference(s);
        const double* src = which == 0 ? s->ref->mass.data() : s->ref->stiff.data() + (size_t)(which - 1) * n * n;
        std::copy(src, src + (size_t)n * n, dense);
    });
}

tsem_status tsem_assemble(tsem_space s, int32_t which, tsem_csr* out) {
    REQUIRE(s && out, "null argument");
    REQUIRE(which == 0 || which == 1, "which must be 0 (stiffness) or 1 (mass)");
    *out = nullptr;
    return guard([&] {
        auto A = std::make_unique<tsem_csr_s>();
        space_assemble(s, which, A->m);
        A->device = s->device;
        TSEM_CUDA(cudaStreamCreateWithFlags(&A->stream, cudaStreamNonBlocking));
        *out = A.release();
    });
}

tsem_status tsem_csr_info(tsem_csr A, int64_t* n, int64_t* nnz) {
    REQUIRE(A, "null argument");
    if (n) *n = A->m.n;
    if (nnz) *nnz = A->m.nnz;
    return TSEM_OK;
}

tsem_status tsem_csr_export(tsem_csr A, int64_t* rowptr, int32_t* col, double* val) {
    REQUIRE(A, "null argument");
    return guard([&] {
        if (rowptr) A->m.rowptr.download(rowptr, A->m.n + 1, A->stream);
        if (col) A->m.col.download(col, A->m.nnz, A->stream);
        if (val) A->m.val.download(val, A->m.nnz, A->stream);
        TSEM_CUDA(cudaStreamSynchronize(A->stream));
    });
}

tsem_status tsem_csr_import(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, tsem_csr* out) {
    REQUIRE(out && rowptr && col && val && n > 0, "null argument");
    REQUIRE(rowptr[0] == 0, "rowptr[0] must be 0");
    for (int64_t r = 0; r < n; ++r) {
        REQUIRE(rowptr[r + 1] > rowptr[r], "every row needs its diagonal");
        REQUIRE(col[rowptr[r]] == r, "the diagonal must come first in every row");
    }
    for (int64_t k = 0; k < rowptr[n]; ++k) REQUIRE(col[k] >= 0 && col[k] < n, "column index out of range");
    *out = nullptr;
    return guard([&] {
        auto A = std::make_unique<tsem_csr_s>();
        ensure_stream(&A->stream, &A->device);
        A->m.n = n;
        A->m.nnz = rowptr[n];
        A->m.rowptr.upload(rowptr, n + 1, A->stream);
        A->m.col.upload(col, A->m.nnz, A->stream);
        A->m.val.upload(val, A->m.nnz, A->stream);
        A->m.refresh_diag(A->stream);
        TSEM_CUDA(cudaStreamSynchronize(A->stream));
        *out = A.release();
    });
}

tsem_status tsem_csr_copy(tsem_csr A, tsem_csr* out) {
    REQUIRE(A && out, "null argument");
    *out = nullptr;
    return guard([&] {
        auto B = std::make_unique<tsem_csr_s>();
        ensure_stream(&B->stream, &B->device);
        B->m.n = A->m.n;
        B->m.nnz = A->m.nnz;
        TSEM_CUDA(cudaStreamSynchronize(A->stream));
        B->m.rowptr.alloc(A->m.n + 1);
        B->m.col.alloc(A->m.nnz);
        B->m.val.alloc(A->m.nnz);
        TSEM_CUDA(cudaMemcpyAsync(B->m.rowptr.p, A->m.rowptr.p, (A->m.n + 1) * sizeof(int64_t), cudaMemcpyDeviceToDevice, B->stream));
        TSEM_CUDA(cudaMemcpyAsync(B->m.col.p, A->m.col.p, A->m.nnz * sizeof(int), cudaMemcpyDeviceToDevice, B->stream));
        TSEM_CUDA(cudaMemcpyAsync(B->m.val.p, A->m.val.p, A->m.nnz * sizeof(double), cudaMemcpyDeviceToDevice, B->stream));
        B->m.refresh_diag(B->stream);
        TSEM_CUDA(cudaStreamSynchronize(B->stream));
        *out = B.release();
    });
}

void tsem_csr_destroy(tsem_csr A) {
    if (!A) return;
    cudaStream_t st = A->stream;
    if (st) cudaStreamSynchronize(st);
    delete A;
    if (st) cudaStreamDestroy(st);
    trace_mark("csr_destroy");
}

tsem_status tsem_csr_spmv(tsem_csr A, const double* x, double* y, int32_t device, void* stream) {
    REQUIRE(A && x && y, "null argument");
    return guard([&] {
        cudaStream_t s = pick(stream, A->stream);
        spmv_autotune(A->m, s);
        if (device) {
            csr_spmv(A->m, x, y, s);
            TSEM_CUDA(cudaStreamSynchronize(s));
        } else {
            DBuf<double> dx, dy(A->m.n);
            dx.upload(x, A->m.n, s);
            csr_spmv(A->m, dx.p, dy.p, s);
            dy.download(y, A->m.n, s);
            TSEM_CUDA(cudaStreamSynchronize(s));
        }
    });
}

tsem_status tsem_csr_spmv_tuning(tsem_csr A, int32_t* shape, float* ms, float* shape_ms, double* shape_err,
                                 int32_t cap, int32_t* count) {
    REQUIRE(A && shape && ms && count, "null argument");
    REQUIRE(cap >= 0, "bad buffer size");
    return guard([&] {
        *shape = A->m.spmv_variant;
        *ms = A->m.spmv_ms;
        const auto& t = A->m.spmv_shape_ms;
        const auto& e = A->m.spmv_shape_err;
        *count = (int32_t)t.size();
        for (int32_t i = 0; i < cap && i < (int32_t)t.size(); ++i) {
            if (shape_ms) shape_ms[i] = t[i];
            if (shape_err) shape_err[i] = i < (int32_t)e.size() ? e[i] : 0.0;
        }
    });
}

tsem_status tsem_rhs(tsem_space s, const double* f_qp, double* r) {
    REQUIRE(s && f_qp && r, "null argument");
    return guard([&] { rhs(s, f_qp, r); });
}

tsem_status tsem_neumann(tsem_space s, double* r, const double* g, int32_t flag) {
    REQUIRE(s && r && g, "null argument");
    return guard([&] { neumann(s, r, g, flag); });
}

tsem_status tsem_dirichlet(tsem_space s, tsem_csr A, double* r, const double* uv, const double* ue, const double* uf,
                           int32_t modify, int32_t flag) {
    REQUIRE(s && A && r && uv && ue && uf, "null argument");
    return guard([&] {
        TSEM_CUDA(cudaStreamSynchronize(A->stream));
        dirichlet(s, A->m, r, uv, ue, uf, modify != 0, flag);
    });
}

tsem_status tsem_zero_bc(tsem_space s, tsem_csr A, double* r, int32_t flag) {
    REQUIRE(s, "null argument");
    return guard([&] {
        if (A) TSEM_CUDA(cudaStreamSynchronize(A->stream));
        zero_bc(s, A ? &A->m : nullptr, r, flag);
    });
}

tsem_status tsem_errors(tsem_space s, const double* sol, const double* uq, const double* guq, double* out) {
    REQUIRE(s && sol && uq && guq && out, "null argument");
    return guard([&] { errors(s, sol, uq, guq, out); });
}

tsem_status tsem_assemble_potential(tsem_space s, const double* v_qp, tsem_csr* inout) {
    REQUIRE(s && v_qp && inout, "null argument");
    return guard([&] {
        if (*inout) {
            TSEM_CUDA(cudaStreamSynchronize((*inout)->stream));
            assemble_potential(s, v_qp, (*inout)->m);
            return;
        }
        auto A = std::make_unique<tsem_csr_s>();
        assemble_potential(s, v_qp, A->m);
        A->device = s->device;
        TSEM_CUDA(cudaStreamCreateWithFlags(&A->stream, cudaStreamNonBlocking));
        *inout = A.release();
    });
}

tsem_status tsem_interpolation(tsem_space s, const double* u_v, const double* u_e, const double* u_f,
                               const double* u_qp, double* out) {
    REQUIRE(s && u_v && u_e && u_f && u_qp && out, "null argument");
    return guard([&] { interpolation(s, u_v, u_e, u_f, u_qp, out); });
}

tsem_status tsem_eval_qp(tsem_space s, const double* sol, double* out) {
    REQUIRE(s && sol && out, "null argument");
    return guard([&] { eval_qp(s, sol, out); });
}

tsem_status tsem_eval_qp_device(tsem_space s, const double* sol, double* out, void* stream) {
    REQUIRE(s && sol && out, "null argument");
    return guard([&] { eval_qp_device(s, sol, out, pick(stream, s->stream)); });
}

tsem_status tsem_density(tsem_space s, const double* states, int32_t k, const double* occ, double* out) {
    REQUIRE(s && states && occ && out, "null argument");
    return guard([&] { density(s, states, k, occ, out); });
}

tsem_status tsem_density_device(tsem_space s, const double* states, int32_t k, const double* occ, double* out,
                                void* stream) {
    REQUIRE(s && states && occ && out, "null argument");
    return guard([&] { density_device(s, states, k, occ, out, pick(stream, s->stream)); });
}

tsem_status tsem_density_l2_difference(tsem_space s, const double* u, const double* v, int32_t k, const double* occ,
                                       double* out) {
    REQUIRE(s && u && v && occ && out, "null argument");
    return guard([&] { *out = density_l2_difference(s, u, v, k, occ); });
}

tsem_status tsem_rhs_device(tsem_space s, const double* f_qp, double* r, void* stream) {
    REQUIRE(s && f_qp && r, "null argument");
    return guard([&] { rhs_device(s, f_qp, r, pick(stream, s->stream)); });
}

tsem_status tsem_assemble_potential_device(tsem_space s, const double* v_qp, tsem_csr* inout, void* stream) {
    REQUIRE(s && v_qp && inout, "null argument");
    return guard([&] {
        cudaStream_t st = pick(stream, s->stream);
        if (*inout) {
            TSEM_CUDA(cudaStreamSynchronize((*inout)->stream));
            assemble_potential_device(s, v_qp, (*inout)->m, st);
            return;
        }
        auto A = std::make_unique<tsem_csr_s>();
        assemble_potential_device(s, v_qp, A->m, st);
        A->device = s->device;
        TSEM_CUDA(cudaStreamCreateWithFlags(&A->stream, cudaStreamNonBlocking));
        *inout = A.release();
    });
}

tsem_status tsem_csr_add(tsem_csr dst, double alpha, tsem_csr src) {
    REQUIRE(dst && src, "null argument");
    return guard([&] {
        TSEM_CUDA(cudaStreamSynchronize(src->stream));
        csr_axpy(dst->m, alpha, src->m, dst->stream);
    });
}

tsem_status tsem_solver_create(tsem_csr A, const int32_t* sum_dof, int32_t p, const tsem_solver_opts* opts,
                               tsem_solver* out) {
    REQUIRE(A && opts && out, "null argument");
    REQUIRE(opts->precond != 4 || sum_dof, "p-multigrid needs sum_dof");
    *out = nullptr;
    return guard([&] {
        auto sv = std::make_unique<tsem_solver_s>();
        ensure_stream(&sv->stream, &sv->device);
        TSEM_CUDA(cudaStreamSynchronize(A->stream));
        std::vector<int> sd;
        if (sum_dof) sd.assign(sum_dof, sum_dof + A->m.n);
        sv->impl = std::make_unique<Solver>(&A->m, *opts, sd, p, sv->stream);
        TSEM_CUDA(cudaStreamSynchronize(sv->stream));
        *out = sv.release();
    });
}

void tsem_solver_destroy(tsem_solver sv) {
    if (!sv) return;
    cudaStream_t st = sv->stream;
    if (st) cudaStreamSynchronize(st);
    trace_mark("solver_sync");
    delete sv;
    trace_mark("solver_delete");
    if (st) cudaStreamDestroy(st);
}

// A caller's host array pinned in place for the duration of a call, so that its
// copies run as DMA at full link speed; when the memory cannot be registered
// (already registered, or not registrable) the copies stay staged.
struct HostPin {
    void* p = nullptr;
    HostPin(const void* ptr, size_t bytes) {
        if (cudaHostRegister(const_cast<void*>(ptr), bytes, cudaHostRegisterDefault) == cudaSuccess)
            p = const_cast<void*>(ptr);
        else
            (void)cudaGetLastError();
    }
    ~HostPin() {
        if (p) cudaHostUnregister(p);
    }
    HostPin(const HostPin&) = delete;
    HostPin& operator=(const HostPin&) = delete;
};

tsem_status tsem_solve_pcg(tsem_solver sv, const double* b, double* x, tsem_stats* st) {
    REQUIRE(sv && b && x, "null argument");
    tsem_stats local{};
    tsem_status rc = guard([&] {
        if (sv->mixed) {
            MixedSolver& S = *sv->mixed;
            const int64_t n = S.A->n;
            if (sv->hb.n < (size_t)n) { sv->hb.alloc(n); sv->hx.alloc(n); }
            HostPin pb(b, (size_t)n * sizeof(double)), px(x, (size_t)n * sizeof(double));
            trace_mark("pin");
            sv->hb.upload(b, n, sv->stream);
            sv->hx.upload(x, n, sv->stream);
            S.solve(sv->hb.p, sv->hx.p, &local, sv->stream);
            trace_mark("pcg");
            sv->hx.download(x, n, sv->stream);
            TSEM_CUDA(cudaStreamSynchronize(sv->stream));
            return;
        }
        Solver& S = *sv->impl;
        const int64_t n = S.A->n;
        HostPin pb(b, (size_t)n * sizeof(double)), px(x, (size_t)n * sizeof(double));
        S.b.upload(b, n, sv->stream);
        S.x.upload(x, n, sv->stream);
        S.solve(S.b.p, S.x.p, &local, sv->stream);
        S.x.download(x, n, sv->stream);
        TSEM_CUDA(cudaStreamSynchronize(sv->stream));
    });
    if (st) *st = local;
    if (rc != TSEM_OK) return rc;
    return (tsem_status)local.status;
}

tsem_status tsem_solve_pcg_device(tsem_solver sv, const double* b, double* x, tsem_stats* st, void* stream) {
    REQUIRE(sv && b && x, "null argument");
    tsem_stats local{};
    tsem_status rc = guard([&] {
        cudaStream_t s = pick(stream, sv->stream);
        if (sv->mixed) sv->mixed->solve(b, x, &local, s);
        else sv->impl->solve(b, x, &local, s);
    });
    if (st) *st = local;
    if (rc != TSEM_OK) return rc;
    return (tsem_status)local.status;
}

static tsem_status lobpcg_common(tsem_solver sv, tsem_csr Aop, tsem_csr M, int32_t k, int32_t n_want, double* X,
                                 bool device, double* lambda, double tol, int32_t max_it, tsem_stats* st, void* stream) {
    REQUIRE(sv && M && X && lambda, "null argument");
    tsem_stats local{};
    tsem_status rc = guard([&] {
        if (Aop) TSEM_CUDA(cudaStreamSynchronize(Aop->stream));
        const DevCsr& A = Aop ? Aop->m : sv->mixed ? *sv->mixed->A : *sv->impl->A;
        if (A.n != (sv->mixed ? sv->mixed->A->n : sv->impl->A->n))
            throw Error(TSEM_INVALID, "operator and preconditioner differ in size");
        cudaStream_t s = pick(stream, sv->stream);
        TSEM_CUDA(cudaStreamSynchronize(M->stream));
        const int64_t n = A.n;
        DBuf<double> dX;
        double* Xd = X;
        std::unique_ptr<HostPin> pin;
        if (!device) {
            pin = std::make_unique<HostPin>(X, (size_t)n * k * sizeof(double));
            dX.upload(X, (size_t)n * k, s);
            Xd = dX.p;
        }
        LobpcgResult r = lobpcg(A, M->m, sv->impl.get(), sv->mixed.get(), k, n_want, Xd, lambda, tol, max_it, s);
        if (!device) {
            dX.download(X, (size_t)n * k, s);
            TSEM_CUDA(cudaStreamSynchronize(s));
        }
        local.iterations = r.iterations;
        local.status = r.status;
        local.residual_rel = r.residual;
        local.device_ms = r.device_ms;
        local.init_l1 = r.jacobi_sweeps;
    });
    if (st) *st = local;
    if (rc != TSEM_OK) return rc;
    return (tsem_status)local.status;
}

tsem_status tsem_solve_lobpcg(tsem_solver sv, tsem_csr M, int32_t k, int32_t n_want, double* X, double* lambda,
                              double tol, int32_t max_it, tsem_stats* st) {
    return lobpcg_common(sv, nullptr, M, k, n_want, X, false, lambda, tol, max_it, st, nullptr);
}

tsem_status tsem_solve_lobpcg_pencil(tsem_solver precond, tsem_csr A, tsem_csr M, int32_t k, int32_t n_want, double* X,
                                     double* lambda, double tol, int32_t max_it, tsem_stats* st) {
    REQUIRE(A, "null argument");
    return lobpcg_common(precond, A, M, k, n_want, X, false, lambda, tol, max_it, st, nullptr);
}

tsem_status tsem_solve_lobpcg_device(tsem_solver sv, tsem_csr M, int32_t k, int32_t n_want, double* X,
                                     double* lambda, double tol, int32_t max_it, tsem_stats* st, void* stream) {
    return lobpcg_common(sv, nullptr, M, k, n_want, X, true, lambda, tol, max_it, st, stream);
}

tsem_status tsem_solve_pmg(tsem_solver sv, const double* b, double* x, double tol, int32_t max_step, tsem_stats* st) {
    REQUIRE(sv && b && x, "null argument");
    REQUIRE(sv->impl && sv->impl->pmg, "solver has no p-multigrid preconditioner");
    tsem_stats local{};
    tsem_status rc = guard([&] {
        Solver& S = *sv->impl;
        const int64_t n = S.A->n;
        DBuf<double> db, dx;
        db.upload(b, n, sv->stream);
        dx.upload(x, n, sv->stream);
        S.solve_pmg(db.p, dx.p, tol, max_step, &local, sv->stream);
        dx.download(x, n, sv->stream);
        TSEM_CUDA(cudaStreamSynchronize(sv->stream));
    });
    if (st) *st = local;
    if (rc != TSEM_OK) return rc;
    return (tsem_status)local.status;
}

tsem_status tsem_pmg_vcycle(tsem_solver sv, double* x, const double* r) {
    REQUIRE(sv && x && r, "null argument");
    REQUIRE(sv->impl && sv->impl->pmg, "solver has no p-multigrid preconditioner");
    return guard([&] {
        Solver& S = *sv->impl;
        const int64_t n = S.A->n;
        S.r.upload(r, n, sv->stream);
        S.y.upload(x, n, sv->stream);
        S.pmg->vcycle(S.y.p, S.r.p, nullptr, sv->stream);
        S.y.download(x, n, sv->stream);
        TSEM_CUDA(cudaStreamSynchronize(sv->stream));
    });
}

tsem_status tsem_solver_create_mixed(tsem_space s, tsem_csr A, int32_t dirichlet_flag, const tsem_solver_opts* opts,
                                     tsem_solver* out) {
    REQUIRE(s && A && opts && out, "null argument");
    *out = nullptr;
    return guard([&] {
        auto sv = std::make_unique<tsem_solver_s>();
        ensure_stream(&sv->stream, &sv->device);
        TSEM_CUDA(cudaStreamSynchronize(A->stream));
        sv->mixed = std::make_unique<MixedSolver>(s, &A->m, dirichlet_flag, *opts, sv->stream);
        if (opts->inner_tol > 0) sv->mixed->inner_tol = opts->inner_tol;
        TSEM_CUDA(cudaStreamSynchronize(sv->stream));
        *out = sv.release();
    });
}

tsem_status tsem_mf_apply(tsem_solver sv, int32_t level, int32_t low_precision, const double* x, double* y,
                          int64_t* level_n) {
    REQUIRE(sv && sv->mixed, "not a mixed solver");
    auto& op = sv->mixed->op;
    REQUIRE(level >= 0 && level < (int)op.levels.size(), "level out of range");
    const int64_t n = op.levels[level].n;
    if (level_n) *level_n = n;
    if (!x || !y) return TSEM_OK;
    return guard([&] {
        std::vector<float> xf(x, x + n), yf(n);
        DBuf<float> dx, dy(n);
        dx.upload(xf, sv->stream);
        op.apply(level, dx.p, dy.p, sv->stream, low_precision != 0);
        dy.download(yf.data(), n, sv->stream);
        TSEM_CUDA(cudaStreamSynchronize(sv->stream));
        for (int64_t i = 0; i < n; ++i) y[i] = yf[i];
    });
}

tsem_status tsem_mf_apply_device(tsem_solver sv, int32_t level, int32_t low_precision, const float* x, float* y,
                                 void* stream) {
    REQUIRE(sv && sv->mixed && x && y, "not a mixed solver or null argument");
    auto& op = sv->mixed->op;
    REQUIRE(level >= 0 && level < (int)op.levels.size(), "level out of range");
    return guard([&] { op.apply(level, x, y, pick(stream, sv->stream), low_precision != 0); });
}

tsem_status tsem_mf_vcycle_device(tsem_solver sv, int32_t ncol, const float* r, float* z, void* stream) {
    REQUIRE(sv && sv->mixed && r && z, "not a mixed solver or null argument");
    REQUIRE(ncol >= 1, "ncol must be at least 1");
    return guard([&] { sv->mixed->vcycle_graph(r, z, pick(stream, sv->stream), ncol); });
}

tsem_status tsem_mf_profile(tsem_solver sv, int32_t level, int32_t low_precision, int32_t reps, double* out) {
    REQUIRE(sv && sv->mixed && out && reps >= 0, "not a mixed solver or bad argument");
    auto& op = sv->mixed->op;
    REQUIRE(level >= 0 && level < (int)op.levels.size(), "level out of range");
    return guard([&] {
        const int64_t n = op.levels[level].n;
        DBuf<float> x(n), y(n);
        std::vector<float> h(n);
        for (int64_t i = 0; i < n; ++i) h[i] = (float)((i * 7919) % 1000) * 1e-3f - 0.5f;
        x.upload(h, sv->stream);
        op.profile(level, low_precision != 0, reps, x.p, y.p, sv->stream, out);
        TSEM_CUDA(cudaStreamSynchronize(sv->stream));
    });
}

static_assert(TSEM_NOALLOC_SCRATCH_BYTES == kNoAllocScratchBytes, "scratch size of the header and the library differ");

// ------------------------------------------------------------ batched solves
tsem_status tsem_solve_batch(const tsem_solver* sv, int32_t n, const double* const* b, double* const* x, int32_t device,
                             void* stream, tsem_stats* st) {
    REQUIRE(sv && b && x && n >= 1, "null argument or empty batch");
    for (int i = 0; i < n; ++i) {
        REQUIRE(sv[i] && sv[i]->mixed && b[i] && x[i], "not a mixed solver or null argument");
        for (int j = 0; j < i; ++j) REQUIRE(sv[j] != sv[i], "a solver appears twice in the batch");
    }
    std::vector<BatchItem> items(n);
    tsem_status rc = guard([&] {
        int dev = -1;
        TSEM_CUDA(cudaGetDevice(&dev));
        for (int i = 0; i < n; ++i)
            if (sv[i]->device != dev) throw Error(TSEM_INVALID, "every solver of a batch must be on the current device");
        cudaStream_t s = pick(stream, sv[0]->stream);
        std::vector<std::unique_ptr<HostPin>> pins;
        for (int i = 0; i < n; ++i) {
            TSEM_CUDA(cudaStreamSynchronize(sv[i]->stream));
            MixedSolver& S = *sv[i]->mixed;
            const int64_t m = S.A->n;
            items[i].S = &S;
            if (device) {
                items[i].b = b[i];
                items[i].x = x[i];
                continue;
            }
            // host arrays staged through the solver's buffers
            if (sv[i]->hb.n < (size_t)m) { sv[i]->hb.alloc(m); sv[i]->hx.alloc(m); }
            pins.push_back(std::make_unique<HostPin>(b[i], (size_t)m * sizeof(double)));
            pins.push_back(std::make_unique<HostPin>(x[i], (size_t)m * sizeof(double)));
            sv[i]->hb.upload(b[i], m, s);
            sv[i]->hx.upload(x[i], m, s);
            items[i].b = sv[i]->hb.p;
            items[i].x = sv[i]->hx.p;
        }
        solve_batch(items, s);
        if (!device)
            for (int i = 0; i < n; ++i) sv[i]->hx.download(x[i], items[i].S->A->n, s);
        TSEM_CUDA(cudaStreamSynchronize(s));
    });
    if (st)
        for (int i = 0; i < n; ++i) st[i] = items[i].stats;
    if (rc != TSEM_OK) return rc;
    for (int i = 0; i < n; ++i)
        if (items[i].stats.status != TSEM_OK) return (tsem_status)items[i].stats.status;
    return TSEM_OK;
}

// ------------------------------------------------------------- continuous batching
struct tsem_batch_s {
    std::unique_ptr<BatchEngine> eng;
    cudaStream_t stream = nullptr;
    int device = 0;
    std::mutex poll_mu;                                   // one poll (engine round) at a time
    std::mutex mu;                                        // guards the fields below
    int64_t last = 0;
    struct Job {
        int64_t ticket;
        BatchItem item;
        int64_t eng_ticket = 0;
    };
    std::deque<std::unique_ptr<Job>> incoming;            // submitted, not yet in the engine
    std::vector<std::unique_ptr<Job>> running;            // in the engine
    std::deque<std::unique_ptr<Job>> finished;            // retired, not yet reported
    std::vector<int64_t> cancels;                         // tickets to cancel at the next poll
};

tsem_status tsem_batch_create(void* stream, tsem_batch* out) {
    REQUIRE(out, "null argument");
    *out = nullptr;
    return guard([&] {
        auto bt = std::make_unique<tsem_batch_s>();
        if (stream) {
            TSEM_CUDA(cudaGetDevice(&bt->device));
            bt->stream = (cudaStream_t)stream;
        } else {
            ensure_stream(&bt->stream, &bt->device);
        }
        bt->eng = std::make_unique<BatchEngine>(bt->stream);
        *out = bt.release();
    });
}

void tsem_batch_destroy(tsem_batch bt) { delete bt; }

tsem_status tsem_batch_submit(tsem_batch bt, tsem_solver sv, const double* b, double* x, int64_t* ticket) {
    REQUIRE(bt && sv && sv->mixed && b && x && ticket, "null argument or not a mixed solver");
    REQUIRE(sv->device == bt->device, "the solver and the batch are on different devices");
    std::lock_guard<std::mutex> lock(bt->mu);
    for (auto& j : bt->incoming)
        if (j->item.S == sv->mixed.get()) return fail(TSEM_INVALID, "the solver already has a system in the batch");
    for (auto& j : bt->running)
        if (j->item.S == sv->mixed.get()) return fail(TSEM_INVALID, "the solver already has a system in the batch");
    auto j = std::make_unique<tsem_batch_s::Job>();
    j->ticket = ++bt->last;
    j->item.S = sv->mixed.get();
    j->item.b = b;
    j->item.x = x;
    *ticket = j->ticket;
    bt->incoming.push_back(std::move(j));
    return TSEM_OK;
}

tsem_status tsem_batch_cancel(tsem_batch bt, int64_t ticket) {
    REQUIRE(bt, "null argument");
    std::lock_guard<std::mutex> lock(bt->mu);
    bt->cancels.push_back(ticket);
    return TSEM_OK;
}

tsem_status tsem_batch_poll(tsem_batch bt, int32_t cap, int64_t* tickets, tsem_stats* stats, int32_t* n_done,
                            int32_t* n_in_flight) {
    REQUIRE(bt && n_done && cap >= 0 && (cap == 0 || (tickets && stats)), "null argument");
    *n_done = 0;
    return guard([&] {
        std::lock_guard<std::mutex> one_poll(bt->poll_mu);   // the engine is driven by one thread at a time
        TSEM_CUDA(cudaSetDevice(bt->device));
        {
            std::lock_guard<std::mutex> lock(bt->mu);
            while (!bt->incoming.empty()) {
                auto j = std::move(bt->incoming.front());
                bt->incoming.pop_front();
                j->eng_ticket = bt->eng->submit(&j->item);
                bt->running.push_back(std::move(j));
            }
            for (int64_t t : bt->cancels)
                for (auto& j : bt->running)
                    if (j->ticket == t) bt->eng->cancel(j->eng_ticket);
            bt->cancels.clear();
        }
        auto done = bt->eng->round();
        std::lock_guard<std::mutex> lock(bt->mu);
        for (auto& d : done)
            for (auto it = bt->running.begin(); it != bt->running.end(); ++it)
                if ((*it)->eng_ticket == d.first) {
                    bt->finished.push_back(std::move(*it));
                    bt->running.erase(it);
                    break;
                }
        while (*n_done < cap && !bt->finished.empty()) {
            tickets[*n_done] = bt->finished.front()->ticket;
            stats[*n_done] = bt->finished.front()->item.stats;
            bt->finished.pop_front();
            ++*n_done;
        }
        if (n_in_flight)
            *n_in_flight = (int32_t)(bt->incoming.size() + bt->running.size() + bt->finished.size());
    });
}

tsem_status tsem_debug_bounds(int32_t shrink, int32_t* code, int64_t* index, int32_t* checked) {
    return guard([&] {
        int c = 0;
        long long i = 0;
        const bool on = bounds_check(shrink, &c, &i);
        if (code) *code = c;
        if (index) *index = (int64_t)i;
        if (checked) *checked = on ? 1 : 0;
    });
}

tsem_status tsem_debug_wait_limit(int64_t polls) {
    return guard([&] { set_wait_polls((long long)polls); });
}

tsem_status tsem_mf_apply_device_noalloc(tsem_solver sv, int32_t level, const float* x, float* y, void* stream) {
    REQUIRE(sv && sv->mixed && x && y, "not a mixed solver or null argument");
    auto& op = sv->mixed->op;
    REQUIRE(level >= 0 && level < (int)op.levels.size(), "level out of range");
    // y is cleared before x is read, so the two vectors may not share any entry
    const uintptr_t xb = (uintptr_t)x, yb = (uintptr_t)y, nbytes = (uintptr_t)op.levels[level].n * sizeof(float);
    REQUIRE(xb + nbytes <= yb || yb + nbytes <= xb, "x and y overlap; this call needs separate input and output");
    return guard([&] {
        int dev = -1;
        TSEM_CUDA(cudaGetDevice(&dev));
        if (dev != sv->device) throw Error(TSEM_INVALID, "the solver's device must be the current device");
        mf_apply_noalloc(op, level, x, y, pick(stream, sv->stream));
    });
}

}  // extern "C"
