// Request loop of the solver service (no TSEMLib counterpart: the reference solves
// one problem per process).  A stream of Poisson and Laplace-eigen requests of
// mixed mesh size and order is replayed at its arrival times; worker threads take
// requests in arrival order as soon as the device-memory budget admits their
// estimated footprint, each on its own CUDA streams, so requests that arrive while
// others run overlap on the device.  The mixed form's Poisson solves of order <= 6
// run continuously batched: every V-cycle step of the systems of one order in
// flight is one launch (tsem_batch_*).  Every request keeps its mesh, operators,
// multigrid hierarchy and Krylov state resident until it retires, then frees them.
//
// Problem of a request (all seeded, identical whether it runs alone or in a mix):
// unit cube, N^3 Kuhn-split sub-cubes with node jitter, order p, homogeneous
// Dirichlet conditions on every face; Poisson right-hand side a sum of eight
// Gaussians a exp(-|x - c|^2 / (2 w^2)); eigen requests ask for the k smallest
// pairs of the Dirichlet Laplacian (block k + guard vectors).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/tsem_gpu.hpp"
#include "common.hpp"

namespace {

using Clock = std::chrono::steady_clock;

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double uniform(uint64_t& s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }
double normal(uint64_t& s) {
    const double u1 = std::max(uniform(s), 1e-300), u2 = uniform(s);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

// unit cube, n^3 sub-cubes of 6 Kuhn tetrahedra (cube-major), interior nodes
// jittered by U(-jitter h, jitter h) per coordinate, boundary coordinates pinned;
// every boundary geometry marked 1
tsem_gpu::Mesh kuhn_mesh(int n, double jitter, uint64_t seed) {
    const int m = n + 1;
    const double h = 1.0 / n;
    std::vector<double> xyz((size_t)m * m * m * 3);
    uint64_t s = seed ^ 0xA5A5A5A5DEADBEEFull;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j)
            for (int k = 0; k < m; ++k) {
                const int ijk[3] = {i, j, k};
                double* p = &xyz[(((size_t)i * m + j) * m + k) * 3];
                for (int a = 0; a < 3; ++a) {
                    const double d = (2.0 * uniform(s) - 1.0) * jitter * h;
                    p[a] = ijk[a] * h + ((ijk[a] == 0 || ijk[a] == n) ? 0.0 : d);
                }
            }
    static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    auto idx = [m](int i, int j, int k) { return (int32_t)(((int64_t)i * m + j) * m + k); };
    std::vector<int32_t> tets;
    tets.reserve((size_t)n * n * n * 24);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k)
                for (auto& pm : perms) {
                    int off[3] = {0, 0, 0};
                    tets.push_back(idx(i, j, k));
                    for (int a = 0; a < 3; ++a) {
                        off[pm[a]] += 1;
                        tets.push_back(idx(i + off[0], j + off[1], k + off[2]));
                    }
                }
    tsem_gpu::Mesh mesh = tsem_gpu::Mesh::from_tets(std::move(xyz), tets);
    // boundary faces belong to one tetrahedron; their vertices and edges are marked too
    std::vector<int> cnt(mesh.nf(), 0);
    for (int32_t f : mesh.tet_f) ++cnt[f];
    for (int32_t f = 0; f < mesh.nf(); ++f) {
        if (cnt[f] != 1) continue;
        mesh.mark_f[f] = 1;
        for (int k = 0; k < 3; ++k) {
            mesh.mark_v[mesh.face_v[(size_t)f * 3 + k]] = 1;
            mesh.mark_e[mesh.face_e[(size_t)f * 3 + k]] = 1;
        }
    }
    return mesh;
}

// estimated device bytes of a request: FP64 CSR stiffness (and mass for eigen
// requests), matrix-free levels and work vectors
double footprint(const tsem_request& r) {
    const double n = std::pow((double)r.order * r.n_cube + 1.0, 3);
    const double nl = (r.order + 1.0) * (r.order + 2.0) * (r.order + 3.0) / 6.0;
    const double E = 6.0 * std::pow((double)r.n_cube, 3);
    const double nnz_row = std::min(n, 1.6 * nl * 1.9);   // measured 69-152 per row for p = 4..6
    const double csr = 12.0 * n * nnz_row * (r.kind == 1 ? 2.0 : 1.0);
    const double mf = E * nl * 24.0 + n * 200.0;
    const double eig = r.kind == 1 ? 6.0 * 3.0 * (r.n_eig + 4) * n * 8.0 : 0.0;
    return 1.3 * (csr + mf + eig) + 64e6;
}

void cuda_ok(cudaError_t e) {
    if (e != cudaSuccess) throw tsem_gpu::Error(TSEM_CUDA_ERROR, cudaGetErrorString(e));
}

// the right-hand side of a Poisson request: a sum of eight Gaussians
struct Gaussians {
    double a[8], c[8][3], w[8];
};

// its values at the element quadrature points, f[e][q] (the points as the space forms
// them: vertex 0 plus the reference coordinates along the edges from it)
__global__ void k_gauss_qp(int E, int nq, const double* __restrict__ xyz, const int* __restrict__ tet,
                           const double* __restrict__ x3, Gaussians g, double* __restrict__ f) {
    const int64_t total = (int64_t)E * nq;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t / nq), q = (int)(t % nq);
        const double* r = x3 + 3 * (size_t)q;
        const int* nd = tet + 4 * (size_t)e;
        double p[3];
        for (int j = 0; j < 3; ++j) {
            const double p0 = xyz[3 * (size_t)nd[0] + j];
            p[j] = p0 + r[0] * (xyz[3 * (size_t)nd[1] + j] - p0) + r[1] * (xyz[3 * (size_t)nd[2] + j] - p0) +
                   r[2] * (xyz[3 * (size_t)nd[3] + j] - p0);
        }
        double v = 0.0;
        for (int k = 0; k < 8; ++k) {
            const double dx = p[0] - g.c[k][0], dy = p[1] - g.c[k][1], dz = p[2] - g.c[k][2];
            v += g.a[k] * exp(-(dx * dx + dy * dy + dz * dz) / (2.0 * g.w[k] * g.w[k]));
        }
        f[t] = v;
    }
}

// device buffers of one request's set-up, freed when it goes out of scope (inside the
// request's allocation scope: from the stream-ordered pool, freed at the request's end)
struct DevTmp {
    std::vector<std::unique_ptr<tsem::DBuf<char>>> p;
    template <class T>
    T* alloc(size_t n) {
        try {
            p.push_back(std::make_unique<tsem::DBuf<char>>(n * sizeof(T)));
        } catch (const tsem::Error& e) {
            throw tsem_gpu::Error(e.status, e.what());
        }
        return (T*)p.back()->p;
    }
};

// opt-in trace of a request's phases (TSEM_SERVE_TRACE=1): one line per request on stderr
bool trace_on() {
    static const bool on = std::getenv("TSEM_SERVE_TRACE") != nullptr;
    return on;
}

struct Job {
    const tsem_request* r;
    tsem_result* out;
};

// Continuous batching of the mixed solves: request threads submit their systems to
// one batch (tsem_batch_*) and wait; one engine thread polls it, so systems of the
// same order from different requests share every V-cycle launch, new ones join at
// the next round and converged ones retire at once.
struct Batch {
    tsem_batch bt = nullptr;
    std::mutex mu;
    std::condition_variable cv;
    std::vector<std::pair<int64_t, tsem_stats>> done;
    int waiting = 0;
    bool stop = false;
    tsem_status failed = TSEM_OK;
    std::thread thr;

    explicit Batch(int dev) {
        tsem_gpu::check(tsem_batch_create(nullptr, &bt));
        thr = std::thread([this, dev] { engine(dev); });
    }
    ~Batch() {
        {
            std::lock_guard<std::mutex> lock(mu);
            stop = true;
        }
        cv.notify_all();
        thr.join();
        tsem_batch_destroy(bt);
    }
    // the statistics of the system (device arrays b, x) once it has retired
    tsem_stats solve(tsem_solver sv, const double* b, double* x) {
        int64_t ticket = 0;
        tsem_gpu::check(tsem_batch_submit(bt, sv, b, x, &ticket));
        std::unique_lock<std::mutex> lock(mu);
        ++waiting;
        cv.notify_all();
        for (;;) {
            for (size_t i = 0; i < done.size(); ++i)
                if (done[i].first == ticket) {
                    const tsem_stats st = done[i].second;
                    done.erase(done.begin() + (long)i);
                    --waiting;
                    return st;
                }
            if (failed != TSEM_OK) {
                --waiting;
                tsem_gpu::check(failed);
            }
            cv.wait(lock);
        }
    }
    void engine(int dev) {
        cudaSetDevice(dev);
        int64_t ids[64];
        tsem_stats sts[64];
        for (;;) {
            {
                std::unique_lock<std::mutex> lock(mu);
                cv.wait(lock, [&] { return stop || waiting > 0; });
                if (stop) return;
            }
            int32_t nd = 0, nf = 0;
            const tsem_status rc = tsem_batch_poll(bt, 64, ids, sts, &nd, &nf);
            std::lock_guard<std::mutex> lock(mu);
            if (rc != TSEM_OK) failed = rc;
            for (int i = 0; i < nd; ++i) done.emplace_back(ids[i], sts[i]);
            if (nd > 0 || rc != TSEM_OK) cv.notify_all();
        }
    }
};

// returns the moment the request's result was ready (before its buffers are freed)
Clock::time_point run_one(const tsem_request& r, const tsem_serve_opts& o, tsem_result& res, Batch* batch) {
    // the request's buffers come from the stream-ordered pool and are freed at its end
    tsem::AllocScope scope;
    const auto t0 = Clock::now();
    // phases of the request and, when traced, the library's inner phases between them
    struct Phases : tsem::TraceSink {
        std::vector<std::pair<const char*, double>> list;
        Clock::time_point last;
        void mark(const char* name) override {
            const auto now = Clock::now();
            list.emplace_back(name, std::chrono::duration<double>(now - last).count());
            last = now;
        }
    } phases;
    phases.last = t0;
    auto mark = [&](const char* name) { phases.mark(name); };
    struct Install {
        tsem::TraceSink* prev;
        explicit Install(tsem::TraceSink* s) : prev(tsem::t_trace) { tsem::t_trace = s; }
        ~Install() { tsem::t_trace = prev; }
    } install(trace_on() ? &phases : tsem::t_trace);
    Clock::time_point ready = t0;
    tsem_gpu::Mesh mesh = kuhn_mesh(r.n_cube, r.jitter, r.seed);
    tsem_mesh d = mesh.desc();
    tsem_space sp = nullptr;
    tsem_csr A = nullptr, M = nullptr;
    tsem_solver sv = nullptr;
    auto cleanup = [&] {
        if (sv) tsem_solver_destroy(sv);
        if (M) tsem_csr_destroy(M);
        if (A) tsem_csr_destroy(A);
        if (sp) tsem_space_destroy(sp);
    };
    try {
        mark("mesh");
        tsem_gpu::check(tsem_space_create(&d, r.order, r.order + 2, &sp));
        int64_t info[15] = {0};
        tsem_gpu::check(tsem_space_info(sp, info));
        const int64_t n = info[0];
        res.n_dof = n;
        mark("space");
        tsem_gpu::check(tsem_assemble(sp, 0, &A));
        mark("assemble");
        std::vector<double> rhs(n, 0.0);
        if (r.kind == 0) {
            // sum of eight Gaussians at the element quadrature points, evaluated on the
            // device from the mesh and the reference points
            uint64_t s = r.seed ^ 0x5EEDF00Dull;
            Gaussians g{};
            for (int k = 0; k < 8; ++k) {
                g.a[k] = normal(s);
                for (int j = 0; j < 3; ++j) g.c[k][j] = uniform(s);
                g.w[k] = 0.05 + 0.15 * uniform(s);
            }
            const int E = (int)info[2], nq = (int)info[4];
            std::vector<double> x3((size_t)nq * 3);
            tsem_gpu::check(tsem_space_quadrature(sp, x3.data(), nullptr, nullptr, nullptr, nullptr, nullptr));
            DevTmp tmp;
            double* dxyz = tmp.alloc<double>((size_t)d.nv * 3);
            int* dtet = tmp.alloc<int>((size_t)E * 4);
            double* dx3 = tmp.alloc<double>((size_t)nq * 3);
            double* df = tmp.alloc<double>((size_t)E * nq);
            double* drhs = tmp.alloc<double>((size_t)n);
            cuda_ok(cudaMemcpy(dxyz, d.xyz, (size_t)d.nv * 3 * sizeof(double), cudaMemcpyHostToDevice));
            cuda_ok(cudaMemcpy(dtet, d.tet_v, (size_t)E * 4 * sizeof(int), cudaMemcpyHostToDevice));
            cuda_ok(cudaMemcpy(dx3, x3.data(), (size_t)nq * 3 * sizeof(double), cudaMemcpyHostToDevice));
            cudaStream_t st = nullptr;
            cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            k_gauss_qp<<<(unsigned)std::min<int64_t>(((int64_t)E * nq + 255) / 256, 152 * 32), 256, 0, st>>>(
                E, nq, dxyz, dtet, dx3, g, df);
            cudaError_t ke = cudaGetLastError();
            tsem_status rc = ke == cudaSuccess ? tsem_rhs_device(sp, df, drhs, st) : TSEM_CUDA_ERROR;
            if (rc == TSEM_OK) ke = cudaMemcpyAsync(rhs.data(), drhs, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st);
            // the stream finishes whatever was queued, also on failure: the buffers are
            // freed at the request's end without a device-wide wait
            const cudaError_t se = cudaStreamSynchronize(st);
            if (ke == cudaSuccess) ke = se;
            cudaStreamDestroy(st);
            cuda_ok(ke);
            tsem_gpu::check(rc);
            mark("rhs");
        }
        tsem_gpu::check(tsem_zero_bc(sp, A, r.kind == 0 ? rhs.data() : nullptr, 1));
        if (r.kind == 1) {
            tsem_gpu::check(tsem_assemble(sp, 1, &M));
            tsem_gpu::check(tsem_zero_bc(sp, M, nullptr, 1));
        }
        tsem_solver_opts so{};
        so.precond = 4;
        so.pmg_order_step = 2;
        so.smooth_steps = 4;
        so.tol_rel = r.tol;
        if (o.plain) {
            std::vector<int32_t> sd(n);
            tsem_gpu::check(tsem_space_sum_dof(sp, sd.data()));
            so.smoother = 1;
            so.max_iter = 5000;
            tsem_gpu::check(tsem_solver_create(A, sd.data(), r.order, &so, &sv));
        } else {
            so.smoother = 2;
            so.max_iter = 40;
            tsem_gpu::check(tsem_solver_create_mixed(sp, A, 1, &so, &sv));
        }
        mark("solver");
        const auto t1 = Clock::now();
        res.setup_s = std::chrono::duration<double>(t1 - t0).count();
        tsem_stats st{};
        std::vector<double> x;
        if (r.kind == 0) {
            x.assign(n, 0.0);
            if (batch && r.order <= 6) {
                // orders up to 6 take the fused-gather tensor-core GEMM on every level: the
                // batch groups them with the other requests' systems of the same order
                DevTmp tmp;
                double* bx = tmp.alloc<double>(2 * (size_t)n);
                cuda_ok(cudaMemcpy(bx, rhs.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
                cuda_ok(cudaMemset(bx + n, 0, (size_t)n * sizeof(double)));
                st = batch->solve(sv, bx, bx + n);
                cuda_ok(cudaMemcpy(x.data(), bx + n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
                if (st.status != TSEM_OK && st.status != TSEM_MAXIT && st.status != TSEM_BREAKDOWN)
                    tsem_gpu::check((tsem_status)st.status);
            } else {
                tsem_status rc = tsem_solve_pcg(sv, rhs.data(), x.data(), &st);
                if (rc != TSEM_OK && rc != TSEM_MAXIT && rc != TSEM_BREAKDOWN) tsem_gpu::check(rc);
            }
            res.residual = st.residual_rel;
        } else {
            const int k = r.n_eig + std::min(4, std::max(2, r.n_eig / 4));   // guard vectors
            x.assign((size_t)n * k, 0.0);
            uint64_t s = r.seed ^ 0xE16E1ull;
            for (auto& v : x) v = 2.0 * uniform(s) - 1.0;
            for (int j = 0; j < k; ++j) tsem_gpu::check(tsem_zero_bc(sp, nullptr, x.data() + (size_t)j * n, 1));
            std::vector<double> lam(k);
            tsem_status rc =
                tsem_solve_lobpcg(sv, M, k, r.n_eig, x.data(), lam.data(), r.tol_eig > 0 ? r.tol_eig : 1e-8, 500, &st);
            if (rc != TSEM_OK && rc != TSEM_MAXIT && rc != TSEM_BREAKDOWN) tsem_gpu::check(rc);
            res.residual = st.residual_rel;
            res.lambda0 = lam[0];
            res.lambda_last = lam[r.n_eig - 1];
            x.resize(n);   // checksum of the first eigenvector
        }
        res.status = st.status;
        res.iterations = st.iterations;
        double s1 = 0.0, s2 = 0.0;
        for (double v : x) { s1 += v; s2 += v * v; }
        res.checksum = s1;
        res.norm2 = s2;
        if (r.x_out && r.kind == 0) std::memcpy(r.x_out, x.data(), (size_t)n * sizeof(double));
        res.solve_s = std::chrono::duration<double>(Clock::now() - t1).count();
        mark("solve");
    } catch (const tsem_gpu::Error& e) {
        res.status = e.status;
    }
    ready = Clock::now();
    cleanup();
    if (trace_on()) {
        mark("free");
        std::string line = "tsem_serve request " + std::to_string(r.id) + " kind " + std::to_string(r.kind) + " N " +
                           std::to_string(r.n_cube) + " p " + std::to_string(r.order) + ":";
        for (auto& ph : phases.list) line += " " + std::string(ph.first) + " " + std::to_string(ph.second);
        std::fprintf(stderr, "%s\n", line.c_str());
    }
    return ready;
}

}  // namespace

extern "C" tsem_status tsem_serve(const tsem_request* reqs, int64_t n_req, const tsem_serve_opts* opts,
                                  tsem_result* results) {
    if (!reqs || !opts || !results || n_req < 0 || opts->workers < 1) return TSEM_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TSEM_NO_DEVICE;
    {
        // the pool keeps what requests free for the next ones instead of returning it
        cudaMemPool_t pool = nullptr;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
    }
    std::vector<int64_t> order(n_req);
    for (int64_t i = 0; i < n_req; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t a, int64_t b) { return reqs[a].arrival_s < reqs[b].arrival_s; });
    for (int64_t i = 0; i < n_req; ++i) {
        std::memset(&results[i], 0, sizeof(tsem_result));
        results[i].id = reqs[i].id;
        results[i].status = TSEM_INVALID;
    }
    std::mutex mu;
    std::condition_variable cv;
    size_t next = 0;         // next request in arrival order not yet started
    double in_use = 0.0;     // admitted footprint
    int running = 0;
    const double budget = opts->memory_budget_bytes > 0 ? opts->memory_budget_bytes : 150e9;
    const auto start = Clock::now();
    auto now_s = [&] { return std::chrono::duration<double>(Clock::now() - start).count(); };
    // the mixed form's Poisson systems go through one continuously batched engine
    std::unique_ptr<Batch> batch;
    if (!opts->plain) {
        try {
            batch = std::make_unique<Batch>(dev);
        } catch (const tsem_gpu::Error& e) {
            return (tsem_status)e.status;
        }
    }

    auto worker = [&] {
        cudaSetDevice(dev);
        for (;;) {
            int64_t i = -1;
            double need = 0.0;
            {
                std::unique_lock<std::mutex> lock(mu);
                for (;;) {
                    if (next >= order.size()) return;
                    const tsem_request& r = reqs[order[next]];
                    const double t = now_s();
                    const double wait = opts->realtime ? r.arrival_s - t : 0.0;
                    need = footprint(r);
                    if (wait > 0) {
                        cv.wait_for(lock, std::chrono::duration<double>(wait));
                        continue;
                    }
                    if (in_use + need <= budget || running == 0) {
                        i = order[next++];
                        in_use += need;
                        ++running;
                        break;
                    }
                    cv.wait(lock);   // memory frees when a request retires
                }
            }
            const tsem_request& r = reqs[i];
            tsem_result& res = results[i];
            const double t_start = now_s();
            const double t_arrive = opts->realtime ? r.arrival_s : 0.0;
            res.queued_s = t_start - t_arrive;
            if (need > budget) {
                res.status = TSEM_OOM_REFUSED;
            } else {
                const Clock::time_point ready = run_one(r, *opts, res, batch.get());
                res.finish_s = std::chrono::duration<double>(ready - start).count();
            }
            if (res.finish_s <= 0.0) res.finish_s = now_s();
            res.latency_s = res.finish_s - t_arrive;
            {
                std::lock_guard<std::mutex> lock(mu);
                in_use -= need;
                --running;
            }
            cv.notify_all();
        }
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < opts->workers; ++w) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    batch.reset();
    {
        // hand the pool's cached memory back to the device once the service ends
        cudaMemPool_t mp = nullptr;
        if (cudaDeviceGetDefaultMemPool(&mp, dev) == cudaSuccess) cudaMemPoolTrimTo(mp, 0);
        cudaGetLastError();
    }
    return TSEM_OK;
}
