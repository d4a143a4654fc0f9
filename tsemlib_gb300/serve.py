"""Request service: replay a stream of Poisson / eigen requests through tsem_serve.

A request is a dict with keys kind ("poisson" | "eigen"), n (sub-cubes per side),
p (order), k (eigen: wanted pairs), jitter, seed, tol, arrival (seconds); see
include/tsem_gpu.h for the problem each describes.  ``stream`` builds the seeded
request mix of the serving benchmark: Poisson arrivals at a given rate, 80 %
Poisson / 20 % eigen (k uniform in 4..32), N uniform in a range, p uniform in a
range, node jitter 0.1 h, tolerance 1e-10.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from ._lib import check, ptr

KINDS = {"poisson": 0, "eigen": 1}


def stream(n_requests, rate, seed=0, n_range=(4, 32), p_range=(2, 8), k_range=(4, 32), eigen_frac=0.2,
           tol=1e-10):
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    out = []
    for i in range(n_requests):
        eig = rng.random() < eigen_frac
        out.append(dict(id=i, kind="eigen" if eig else "poisson", n=int(rng.integers(n_range[0], n_range[1] + 1)),
                        p=int(rng.integers(p_range[0], p_range[1] + 1)),
                        k=int(rng.integers(k_range[0], k_range[1] + 1)) if eig else 0,
                        jitter=0.1, seed=int(rng.integers(1, 2 ** 62)), tol=tol, arrival=float(t[i])))
    return out


def serve(requests, workers=4, plain=False, realtime=True, budget_gb=150.0, outputs=None):
    """Run the requests; returns one result dict per request (input order).
    outputs: optional {request index: float64 array of n_dof} receiving Poisson solutions."""
    n = len(requests)
    reqs = (_lib.Request * n)()
    keep = []
    for i, r in enumerate(requests):
        q = reqs[i]
        q.id = int(r.get("id", i))
        q.kind = KINDS[r["kind"]]
        q.n_cube = int(r["n"])
        q.order = int(r["p"])
        q.n_eig = int(r.get("k", 0))
        q.jitter = float(r.get("jitter", 0.1))
        q.seed = int(r["seed"])
        q.tol = float(r.get("tol", 1e-10))
        q.tol_eig = float(r.get("tol_eig", 0.0))
        q.arrival_s = float(r.get("arrival", 0.0))
        if outputs is not None and i in outputs:
            keep.append(outputs[i])
            q.x_out = outputs[i].ctypes.data
    res = (_lib.Result * n)()
    opts = _lib.ServeOpts(int(workers), int(bool(plain)), int(bool(realtime)), float(budget_gb) * 1e9)
    check(_lib.lib().tsem_serve(reqs, n, opts, res))
    return [dict(res[i].as_dict(), kind=requests[i]["kind"]) for i in range(n)]


def summary(results):
    """DOF-solves/s over the stream and latency percentiles of the finished requests."""
    ok = [r for r in results if r["status"] in ("OK",)]
    lat = np.array([r["latency_s"] for r in ok]) if ok else np.zeros(1)
    span = max(r["finish_s"] for r in results) if results else 0.0
    dofs = sum(r["n_dof"] for r in ok)
    out = {"requests": len(results), "ok": len(ok), "dof_solves_per_s": dofs / span if span > 0 else 0.0,
           "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
           "wall_s": span}
    # the same per kind of request, with the setup, solve and queueing times behind the latency
    for kind in ("poisson", "eigen"):
        rk = [r for r in ok if r.get("kind") == kind]
        if not rk:
            continue
        lk = np.array([r["latency_s"] for r in rk])
        out[kind] = {"ok": len(rk), "p50_s": float(np.percentile(lk, 50)), "p99_s": float(np.percentile(lk, 99)),
                     "mean_setup_s": float(np.mean([r["setup_s"] for r in rk])),
                     "mean_solve_s": float(np.mean([r["solve_s"] for r in rk])),
                     "mean_queued_s": float(np.mean([r["queued_s"] for r in rk]))}
    return out
