"""Benchmark: DOF-solves/s of the TSEM Poisson solve on GB300.

Workload (default): the unit-cube Poisson problem with mixed boundary conditions
(Dirichlet on x = 0, 1; Neumann elsewhere; u = sin(pi x) sin(pi y) sin(pi z) + x^2),
N = 24 Kuhn-split sub-cubes per side (82 944 tetrahedra, node jitter +-0.1h,
seed 2024), order p = 6 (3 048 625 DOFs).  One step = one FP64 CSR PCG solve
with the p-multigrid V-cycle preconditioner (orders 6 -> 4 -> 2 -> 1) to relative
residual 1e-10, operator, hierarchy and right-hand side resident on the device.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line is printed by rank 0.  Under torchrun every rank solves its own
copy of the problem (independent replicas, no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DOF-solves/s & p99 latency, mixed-prec batched vs FP64 CSR, 1 GB300, res\u22641e-10"
DATA = "synthetic (seeded Kuhn mesh, manufactured solution)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=24)
    ap.add_argument("--p", type=int, default=6)
    ap.add_argument("--smooth", type=int, default=4)
    ap.add_argument("--plain-smooth", type=int, default=5)
    ap.add_argument("--inner-tol", type=float, default=1e-6)
    ap.add_argument("--cpu-sample-iters", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="poisson", choices=["poisson", "serve", "ks", "eig"])
    ap.add_argument("--tf32-peak", action="store_true",
                    help="print the measured cuBLAS TF32 GEMM rate (the denominator of the split-TF32 kernel) and exit")
    ap.add_argument("--requests", type=int, default=40)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--workers", type=int, default=4)
    ap.add_argument("--n-range", default="4,16")
    ap.add_argument("--p-range", default="2,6")
    ap.add_argument("--no-plain", action="store_true", help="serve: skip the sequential plain FP64 arm")
    ap.add_argument("--sweep-rates", default="",
                    help="serve: also replay the same stream at these arrival rates (mixed form), e.g. 50,200,500")
    return ap.parse_args()


def problem(n, p, quad_q=None):
    from tsemlib_gb300 import manufactured as mf
    from tsemlib_gb300 import mesh
    m = mesh.kuhn_cube(n, 0.1, 2024)
    mesh.mark_box_boundary(m, [(0, 0.0), (0, 1.0)])
    return m, mf, quad_q or (p + 2)


def workload_config(args, n_dof, tets, nnz, world):
    """The `config` object of both arms' JSON lines (identical for the same workload)."""
    return {"workload": f"poisson_mixed_bc_N{args.n}_p{args.p}", "n_dof": int(n_dof), "tets": int(tets),
            "nnz": int(nnz), "tol_rel": 1e-10, "l2_flush": "inputs larger than L2 (operator data > 129 MB)",
            "parallelism": f"replicas x{world}"}


class Clocks:
    """nvidia-smi sampling while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _time_solves(step, k, stream):
    """Total and per-solve device time of k solves (events on the solve stream)."""
    import torch
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(k + 1)]
    ev[0].record(stream)
    stats = []
    for i in range(k):
        stats.append(step())
        ev[i + 1].record(stream)
    torch.cuda.synchronize()
    per = [ev[i].elapsed_time(ev[i + 1]) for i in range(k)]
    return ev[0].elapsed_time(ev[k]), stats, per


def _max_over_ranks(ms, dev, world):
    """The slowest rank's time: the whole job ends when it does (replicas, one rank per
    GPU; any torch.distributed backend, the tensor on `dev`)."""
    if world <= 1:
        return float(ms)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def _job_rate(units_per_rank, steps, world, ms):
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return units_per_rank * steps * world / (ms / 1e3)


def _latency(per):
    a = np.asarray(per)
    return {"p50_ms": float(np.percentile(a, 50)), "p99_ms": float(np.percentile(a, 99)), "max_ms": float(a.max()),
            "samples": len(per)}


def ours(args, rank, world):
    import torch
    from tsemlib_gb300 import tsem

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    t0 = time.time()
    m, mf, q = problem(args.n, args.p)
    T = tsem.TSEM(args.p, q, m)
    A = T.stiff_matrix.copy()
    b = T.calc_rhs(mf.f_cfg1)
    T.impose_neumann(b, mf.neumann_cfg1, 2)
    T.impose_boundary_condition(A, b, mf.u_cfg1, True, 1)
    n = T.n_dof_total
    nnz = A.nnz
    sd = T.calc_sum_dof()
    # chosen form: FP64 refinement around the FP32 matrix-free p-multigrid PCG
    mixed = tsem.MixedSolver(T, A, 1, order_step=2, smooth=args.smooth, tol_rel=1e-10, inner_tol=args.inner_tol)
    # plain form: the reference's method in FP64 on the assembled CSR
    plain = tsem.TSEMSolver()
    plain.init_PMG(A, args.p, sd, order_step=2, smoother="chebyshev")
    setup_s = time.time() - t0
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    b_d = torch.from_numpy(b).to(dev)
    x_d = torch.zeros(n, dtype=torch.float64, device=dev)

    def step_mixed():
        x_d.zero_()
        return mixed.solve_device(x_d.data_ptr(), b_d.data_ptr(), stream=stream.cuda_stream)

    def step_plain():
        x_d.zero_()
        return plain.solve_PCG_device(A, x_d.data_ptr(), b_d.data_ptr(), tol_rel=1e-10, flag_preconditioner=4,
                                      var=args.plain_smooth, max_step=2000, stream=stream.cuda_stream)

    for _ in range(args.warmup):
        step_mixed()
    torch.cuda.synchronize()
    # inputs (operator data of several GB) exceed the 129 MB L2: no flush needed between steps
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = tsem.kernel_launches()
    torch.cuda.nvtx.range_push("timed")
    with Clocks(dev.index) as clk:
        ms, stats, per = _time_solves(step_mixed, args.steps, stream)
    torch.cuda.nvtx.range_pop()
    launches = tsem.kernel_launches() - launches0
    if world > 1:
        torch.distributed.barrier()
    ms = _max_over_ranks(ms, dev, world)
    value = _job_rate(n, args.steps, world, ms)
    x = x_d.cpu().numpy()
    rel = float(np.linalg.norm(A.vmult(x) - b) / np.linalg.norm(b))
    l2, h1 = T.calc_errors(x, mf.u_cfg1, mf.grad_cfg1)

    # plain FP64 CSR form on the same problem
    for _ in range(max(1, args.warmup // 2)):
        step_plain()
    ms_plain, st_plain, per_plain = _time_solves(step_plain, args.steps, stream)
    x_plain = x_d.cpu().numpy()
    plain_value = n * args.steps / (ms_plain / 1e3)

    # the reference's exact method on the GPU (lexicographic Gauss-Seidel p-multigrid,
    # two sweeps, as the oracle runs it): one solve, which also gives the iteration
    # count that scales the CPU baseline's sample (the parity tests check that it
    # equals the oracle's within one)
    gs = tsem.TSEMSolver()
    gs.init_PMG(A, args.p, sd, order_step=2, smoother="gs")

    def step_gs():
        x_d.zero_()
        return gs.solve_PCG_device(A, x_d.data_ptr(), b_d.data_ptr(), tol_rel=1e-10, flag_preconditioner=4,
                                   var=2, max_step=2000, stream=stream.cuda_stream)
    ms_gs, st_gs, _ = _time_solves(step_gs, 1, stream)
    gs_iters = st_gs[0]["iterations"]

    # end to end through the public API with host buffers (chosen form)
    xe = np.zeros(n)
    torch.cuda.synchronize()
    h0 = time.perf_counter()
    for _ in range(args.steps):
        xe[:] = 0.0
        mixed.solve(xe, b)
    h1_ = time.perf_counter()
    e2e = n * args.steps * world / (h1_ - h0)

    # kernels of one matrix-free apply on the fine level (smoother operator: BF16 tensor
    # cores; Krylov operator: split-TF32 tensor cores), timed with CUDA events on the
    # solver's stream
    torch.cuda.nvtx.range_push("kprof")
    kp = mixed.profile(0, True, 20)
    kp32 = mixed.profile(0, False, 20)
    torch.cuda.nvtx.range_pop()

    # FP64 CSR SpMV (outer residual of the chosen form, operator of the plain form)
    y_d = torch.empty_like(x_d)
    for _ in range(3):
        A.vmult_device(x_d.data_ptr(), y_d.data_ptr(), stream.cuda_stream)
    reps = 30
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("spmv")
    s0.record(stream)
    for _ in range(reps):
        A.vmult_device(x_d.data_ptr(), y_d.data_ptr(), stream.cuda_stream)
    s1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    spmv_ms = s0.elapsed_time(s1) / reps
    spmv_shape, _, spmv_shape_ms = A.spmv_tuning()
    bytes_spmv = 12 * nnz + 8 * (n + 1) + 16 * n
    achieved = bytes_spmv / (spmv_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()

    line = {
        "metric": METRIC, "value": value, "unit": "DOF-solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 outer / f32 inner", "data": DATA,
        "config": workload_config(args, n, m.nt, nnz, world),
        "form": "matrix-free mixed precision: FP64 refinement, FP32 PCG + matrix-free p-MG (6-4-2-1)",
        "latency": _latency(per),
        "inner_iterations": [s["iterations"] for s in stats], "outer_iterations": [s["outer"] for s in stats],
        "rel_residual": rel, "l2_error": l2, "h1_error": h1, "setup_s": setup_s,
        "plain_fp64_csr": {"value": plain_value, "unit": "DOF-solves/s", "ms_per_step": ms_plain / args.steps,
                           "latency": _latency(per_plain),
                           "iterations": [s["iterations"] for s in st_plain],
                           "max_abs_diff_vs_chosen": float(np.abs(x_plain - x).max()),
                           "speedup_chosen_over_plain": value / world / plain_value},
        "plain_fp64_csr_gauss_seidel": {"value": n / (ms_gs / 1e3), "unit": "DOF-solves/s", "ms_per_step": ms_gs,
                                        "iterations": gs_iters,
                                        "note": "the oracle's algorithm on the GPU: exact lexicographic Gauss-Seidel "
                                                "p-multigrid, two sweeps"},
        "e2e": {"value": e2e, "unit": "DOF-solves/s", "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 8 * n},
        "roofline": _roofline(kp, peak, peak_kind, (args.n, args.p)),
        "kernels": {
            "k_scatter_t_kStore": _bw(kp["bytes_scatter"], kp["ms_scatter"], peak),
            "k_mf_apply_tcg": dict(_bw(kp["bytes_gemm"], kp["ms_gemm"], peak),
                                   tflops=kp["flops_gemm"] / kp["ms_gemm"] / 1e9,
                                   note="BF16 GEMM with the gather fused in; bytes = indices, x, V, weights"),
            "k_gather_x3": _bw(kp32["bytes_gather"], kp32["ms_gather"], peak),
            "k_mf_apply_x3": {"ms_per_launch": kp32["ms_gemm"],
                              "tflops": kp32["flops_gemm"] / kp32["ms_gemm"] / 1e9,
                              "note": "useful FP32-accurate flops; the tensor cores run three TF32 products"},
            "k_spmv_fp64_csr": dict(_bw(bytes_spmv, spmv_ms, peak), frac=achieved / peak,
                                    launch_shape=spmv_shape, shape_ms=[round(t, 4) for t in spmv_shape_ms]),
        },
        "clocks": clk.summary(),
        "gpu_launches": launches,
    }
    if rank == 0 and not args.no_cpu_baseline:
        rp, c, v = A.arrays()
        line["cpu_baseline"] = cpu_baseline(rp, c, v, b, sd, args, gs_iters)
    return line


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the
# Chebyshev-step scatter of the level-0 apply, from an ncu capture of this bench's
# kernel-timing range ("kprof"), keyed by (N, p)
SCATTER_CHEB_TRAFFIC = {(24, 6): 131921152}


def _bw(nbytes, ms, peak):
    gbs = nbytes / (ms / 1e3) / 1e9
    return {"ms_per_launch": ms, "bytes_per_launch": nbytes, "gbs": gbs, "frac_hbm": gbs / peak}


def _roofline(kp, peak, peak_kind, key):
    """The dominant kernel of the timed solve: the transposed scatter with a Chebyshev
    step fused in (k_scatter_t<unit, kChebStep>, the largest share of the ncu launch
    list), timed on the level-0 smoother apply with its own vectors."""
    achieved = kp["bytes_scatter_cheb"] / (kp["ms_scatter_cheb"] / 1e3) / 1e9
    return {"kernel": "k_scatter_t<1, kChebStep> (level-0 scatter with the Chebyshev step fused in)",
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": SCATTER_CHEB_TRAFFIC.get(key), "peak_source": peak_kind,
            "bytes_per_launch": kp["bytes_scatter_cheb"], "ms_per_launch": kp["ms_scatter_cheb"]}


def _oracle_sample(Ao, b, P, k):
    """Wall time per PCG iteration of the oracle over a k-iteration sample."""
    import oracle
    t0 = time.perf_counter()
    _, st = oracle.pcg(Ao, b, tol=0.0, rel_tol=1e-300, max_step=k - 1, flag=4, pmg=P, smooth=2)
    dt = time.perf_counter() - t0
    return dt / max(st["iterations"], 1), st["iterations"], dt


def _omp_threads():
    """Threads of the oracle's OpenMP loops (all host cores unless OMP_NUM_THREADS says less)."""
    import oracle
    return oracle.get_threads()


def cpu_baseline(rp, c, v, b, sum_dof, args, iters):
    """The oracle's p-multigrid PCG on the host cores: a bounded sample of
    iterations on the same matrix, scaled by the iteration count of the full solve
    (`iters`, measured in this run by the same algorithm on the GPU)."""
    import oracle
    Ao = oracle.Csr.from_arrays(rp, c, v)
    P = oracle.PMG(Ao, args.p, sum_dof, 2)
    cores = _omp_threads()
    per_iter, k, _ = _oracle_sample(Ao, b, P, args.cpu_sample_iters)
    # the same solve on one core: one iteration
    oracle.set_threads(1)
    try:
        per_iter1, k1, _ = _oracle_sample(Ao, b, P, 1)
    finally:
        oracle.set_threads(cores)
    n = len(rp) - 1
    return {"value": n / (per_iter * iters), "unit": "DOF-solves/s", "cores": cores, "kind": "port",
            "sample": f"{k} PCG iterations of the oracle p-MG (V-cycle {args.p}-..-1, 2 Gauss-Seidel sweeps, "
                      f"OpenMP SpMV) on the same CSR, {per_iter:.2f} s/iteration, scaled to the {iters} "
                      f"iterations to 1e-10 of the same algorithm's solve on the GPU in this run",
            "single_core": {"value": n / (per_iter1 * iters), "unit": "DOF-solves/s", "cores": 1,
                            "sample": f"{k1} PCG iteration of the same solve on one thread, "
                                      f"{per_iter1:.2f} s/iteration, scaled the same way"}}


def reference(args):
    """The reference's CPU path as restated by the oracle (TSEMLib itself needs
    AFEPack, deal.II and LAPACKE, none of which exist here): oracle assembly,
    boundary conditions and p-multigrid set-up outside the timed region; one full
    solve to relative residual 1e-10, which gives the iteration count and a whole
    solve's wall time; then every step times a bounded sample of PCG iterations of
    the same solve, scaled by that count."""
    import oracle
    world = int(os.environ.get("WORLD_SIZE", "1"))
    m, mf, q = problem(args.n, args.p)
    t0 = time.time()
    S = oracle.Space(m, args.p, quad_q=q)
    A = S.assemble("stiff")
    b = S.rhs(mf.f_cfg1)
    S.neumann(b, mf.neumann_cfg1, 2)
    S.dirichlet(A, b, mf.u_cfg1, True, 1)
    P = oracle.PMG(A, args.p, S.sum_dof(), 2)
    setup_s = time.time() - t0
    n = A.n
    t0 = time.perf_counter()
    _, st_full = oracle.pcg(A, b, tol=0.0, rel_tol=1e-10, max_step=5000, flag=4, pmg=P, smooth=2)
    full_s = time.perf_counter() - t0
    iters = st_full["iterations"]
    k = args.cpu_sample_iters
    for _ in range(args.warmup):
        _oracle_sample(A, b, P, k)
    per, total = [], 0.0
    for _ in range(args.steps):
        pi, kk, dt = _oracle_sample(A, b, P, k)
        per.append(pi)
        total += dt
    per_iter = float(np.mean(per))
    value = n / (per_iter * iters)
    cores = _omp_threads()
    sample = (f"each step: {k} PCG iterations of the oracle p-MG solve (V-cycle {args.p}-..-1, 2 Gauss-Seidel "
              f"sweeps, OpenMP SpMV) on the oracle-assembled CSR; {per_iter:.2f} s/iteration scaled to the {iters} "
              f"iterations of the full solve to 1e-10 run before the steps ({full_s:.1f} s)")
    return {"metric": METRIC, "value": value, "unit": "DOF-solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA, "impl": "reference",
            "config": workload_config(args, n, m.nt, A.nnz, world),
            "form": "oracle restatement of TSEMLib's FP64 CSR p-MG PCG on the host cores",
            "setup_s": setup_s, "solve_ms_estimate": 1e3 * per_iter * iters,
            "full_solve": {"s": full_s, "iterations": iters,
                           "rel_residual": float(st_full["residual_l2"] / np.linalg.norm(b)),
                           "value": n / full_s, "unit": "DOF-solves/s"},
            "cpu_baseline": {"value": value, "unit": "DOF-solves/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "DOF-solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def serve_workload(args, rank, world):
    """The serving stream: Poisson-process arrivals, 80 % Poisson / 20 % eigen
    (k in 4..32), N and p uniform in the given ranges, jitter 0.1 h, tol 1e-10;
    the mixed matrix-free solver with concurrent requests against the plain FP64
    CSR solver run one request at a time."""
    import torch
    from tsemlib_gb300 import serve
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    nr = tuple(int(v) for v in args.n_range.split(","))
    pr = tuple(int(v) for v in args.p_range.split(","))
    reqs = serve.stream(args.requests, args.rate, seed=2024 + rank, n_range=nr, p_range=pr)
    serve.serve(reqs[:2], workers=2, realtime=False)          # warm-up: module load, first allocations
    with Clocks(torch.cuda.current_device()) as clk:
        res = serve.serve(reqs, workers=args.workers, realtime=True)
    s_mixed = serve.summary(res)
    s_plain = None
    if not args.no_plain:
        res_plain = serve.serve(reqs, workers=1, plain=True, realtime=True)
        s_plain = serve.summary(res_plain)
    sweep = []
    for r in [float(v) for v in args.sweep_rates.split(",") if v.strip()]:
        # the same requests (sizes, seeds) arriving at another rate
        rq = serve.stream(args.requests, r, seed=2024 + rank, n_range=nr, p_range=pr)
        sr = serve.summary(serve.serve(rq, workers=args.workers, realtime=True))
        sweep.append({"rate_per_s": r, "dof_solves_per_s": sr["dof_solves_per_s"], "p50_s": sr["p50_s"],
                      "p99_s": sr["p99_s"], "ok": sr["ok"], "wall_s": sr["wall_s"]})
    line = {
        "metric": METRIC, "value": s_mixed["dof_solves_per_s"] * world, "unit": "DOF-solves/s", "n_gpus": world,
        "steps": args.requests, "warmup": 2, "ms_per_step": 1e3 * s_mixed["wall_s"] / max(1, args.requests),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 outer / f32 inner",
        "data": "synthetic (seeded request stream: Kuhn meshes, Gaussian right-hand sides)",
        "config": {"workload": f"serve_{args.requests}req_rate{args.rate:g}_N{nr[0]}-{nr[1]}_p{pr[0]}-{pr[1]}",
                   "requests": args.requests, "rate_per_s": args.rate, "mix": "80% Poisson / 20% eigen k 4..32",
                   "workers": args.workers, "tol_rel": 1e-10, "parallelism": f"replicas x{world}"},
        "latency": {"p50_s": s_mixed["p50_s"], "p99_s": s_mixed["p99_s"], "ok": s_mixed["ok"]},
        "by_kind": {k: s_mixed[k] for k in ("poisson", "eigen") if k in s_mixed},
        "plain_fp64_csr_sequential": s_plain,
        "speedup_over_plain": (s_mixed["dof_solves_per_s"] / max(s_plain["dof_solves_per_s"], 1e-30)
                               if s_plain else None),
        "clocks": clk.summary(),
    }
    if sweep:
        line["rate_sweep"] = sweep
    return line


def ks_workload(args, rank, world):
    """Helium Kohn-Sham SCF: graded [-10, 10]^3 mesh (10 sub-cubes per half-axis,
    ratio 1.15), p = 5, LDA exchange, mixing 0.3, <= 40 iterations, |dE| < 1e-8."""
    import torch
    from tsemlib_gb300 import ks
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    ks.helium(p=2, n_half=2, max_iter=2)       # warm-up: module load
    with Clocks(torch.cuda.current_device()) as clk:
        out = ks.helium(p=5, n_half=10)
    hist = out.pop("history")
    return {"metric": "Kohn-Sham SCF wall time (helium, LDA exchange, |dE| < 1e-8)", "value": out["scf_s"],
            "unit": "s", "n_gpus": world, "steps": out["iterations"], "warmup": 1,
            "ms_per_step": 1e3 * out["scf_s"] / max(1, out["iterations"]), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 (eigen, Gram, potentials) / f32 preconditioner",
            "data": "synthetic (graded Kuhn mesh, smoothed -2/r nucleus)",
            "config": {"workload": "ks_helium_N20_graded_p5", "n_dof": out["n_dof"], "parallelism": f"replicas x{world}"},
            "result": out, "energies": [h["energy"] for h in hist],
            "lobpcg_iterations": [h["lobpcg_iterations"] for h in hist],
            "phase_s": {k: round(sum(h.get(k, 0.0) for h in hist), 3)
                        for k in ("hamiltonian_s", "lobpcg_s", "density_hartree_s", "density_moments_s",
                                  "rhs_boundary_s", "hartree_solve_s", "hartree_points_s")},
            "hartree_iterations": [h.get("hartree_iterations") for h in hist],
            "clocks": clk.summary()}


def eig_workload(args, rank, world):
    """Laplace eigenpairs (config 3): Dirichlet unit cube, N = 16 Kuhn sub-cubes per side
    (24 576 tets, no jitter), p = 5, block LOBPCG with k = 20 for the lowest 16 pairs
    from a seeded random FP64 block, relative residual 1e-8; the chosen form
    (matrix-free FP32 block V-cycle preconditioner) and the plain form (FP64 V-cycle),
    eigenvalues against pi^2 (i^2 + j^2 + k^2)."""
    import torch
    from tsemlib_gb300 import mesh, tsem
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    n, p, k, want = 16, 5, 20, 16
    m = mesh.mark_all_boundary(mesh.kuhn_cube(n, 0.0, 1))
    T = tsem.TSEM(p, p + 2, m)
    A = T.stiff_matrix.copy()
    M = T.mass_matrix.copy()
    T.impose_zero_boundary_condition(A, None, 1)
    T.impose_zero_boundary_condition(M, None, 1)
    rng = np.random.default_rng(2024 + rank)
    X0 = rng.uniform(-1.0, 1.0, (T.n_dof_total, k))
    for j in range(k):
        c = np.ascontiguousarray(X0[:, j])
        T.impose_zero_boundary_condition(None, c, 1)
        X0[:, j] = c
    analytic = np.sort([np.pi ** 2 * (i * i + j * j + l * l) for i in range(1, 8) for j in range(1, 8)
                        for l in range(1, 8)])[:want]
    mixed = tsem.MixedSolver(T, A, 1, order_step=2)
    plain = tsem.TSEMSolver()
    plain.init_PMG(A, p, T.calc_sum_dof(), order_step=2, smoother="chebyshev")
    runs = {"mixed": lambda Y: mixed.solve_LOBPCG(Y, M, tol=1e-8, max_step=500, n_want=want),
            "plain": lambda Y: plain.solve_LOBPCG(T, Y, A, M, tol=1e-8, max_step=500, n_want=want, smooth_step=4)}
    out = {}
    with Clocks(torch.cuda.current_device()) as clk:
        for name, run in runs.items():
            run(X0.copy())                              # warm-up: graphs, autotuning
            times = []
            torch.cuda.nvtx.range_push(f"eig_{name}")
            for _ in range(max(1, args.steps)):
                t0 = time.perf_counter()
                lam, st = run(X0.copy())
                times.append(time.perf_counter() - t0)
            torch.cuda.nvtx.range_pop()
            out[name] = {"s": float(np.median(times)), "iterations": st["iterations"], "status": st["status"],
                         "jacobi_sweeps_max": st["jacobi_sweeps"],
                         "max_rel_err_vs_analytic": float(np.max(np.abs(lam[:want] - analytic) / analytic))}
    return {"metric": "LOBPCG wall time (16 lowest Laplace eigenpairs, residual < 1e-8)", "value": out["mixed"]["s"],
            "unit": "s", "n_gpus": world, "steps": max(1, args.steps), "warmup": 1,
            "ms_per_step": 1e3 * out["mixed"]["s"], "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 on (hi, lo) f32 pairs (block products, Gram, Ritz combinations, Jacobi), f64 (Rayleigh-Ritz factorisation) / f32 preconditioner",
            "data": "synthetic (seeded random initial block)",
            "config": {"workload": f"laplace_eig_N{n}_p{p}_k{k}_want{want}", "n_dof": T.n_dof_total,
                       "parallelism": f"replicas x{world}"},
            "forms": out, "clocks": clk.summary()}


def tf32_peak():
    """cuBLAS TF32 GEMM throughput (torch.matmul on FP32 with TF32 allowed), square N^3
    products, CUDA events after three warm-ups: the measured TF32 tensor peak."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = True
    out = {}
    for n, reps in ((8192, 20), (16384, 6)):
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        for _ in range(3):
            c = a @ b
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            c = a @ b
        e1.record()
        torch.cuda.synchronize()
        out[str(n)] = 2.0 * n ** 3 / (e0.elapsed_time(e1) / reps / 1e3) / 1e12
        del a, b, c
    return {"tf32_gemm_tflops": out}


def main():
    args = parse()
    if args.tf32_peak:
        print(json.dumps(tf32_peak()))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:          # the other ranks exit without work
            print(json.dumps(reference(args)))
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    work = {"serve": serve_workload, "ks": ks_workload, "eig": eig_workload}.get(args.workload, ours)
    line = work(args, rank, world)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
