"""bench.py's reference arm runs the oracle on the host cores only, so its JSON
line can be checked here without a GPU: one line, the keys and types the bench
contract asks for, and a solve that reached its tolerance."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "3", "--p", "4", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for key, typ in [("metric", str), ("value", float), ("unit", str), ("n_gpus", int), ("steps", int),
                     ("warmup", int), ("ms_per_step", float), ("higher_is_better", bool), ("scaling", str),
                     ("dtype", str), ("data", str), ("config", dict), ("impl", str), ("cpu_baseline", dict),
                     ("e2e", dict)]:
        assert key in d and isinstance(d[key], typ), (key, d.get(key))
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert "workload" in d["config"]
    # the same config object as the GPU arm's for this workload
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    want = bench.workload_config(argparse.Namespace(n=3, p=4), d["config"]["n_dof"], d["config"]["tets"],
                                 d["config"]["nnz"], 1)
    assert d["config"] == want
    # the iteration count that scales the samples comes from a full solve in the same run
    assert d["full_solve"]["iterations"] > 0 and d["full_solve"]["rel_residual"] <= 1e-10
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["cores"] >= 1


def test_cpu_baseline_reports_all_threads_and_one_thread():
    """The CPU baseline times the oracle's p-MG PCG on all host threads and again on
    one thread, and leaves the oracle's thread count as it found it."""
    import argparse
    sys.path.insert(0, ROOT)
    import bench
    import oracle
    m, mf, q = bench.problem(3, 4)
    S = oracle.Space(m, 4, quad_q=q)
    A = S.assemble("stiff")
    b = S.rhs(mf.f_cfg1)
    S.neumann(b, mf.neumann_cfg1, 2)
    S.dirichlet(A, b, mf.u_cfg1, True, 1)
    rp, c, v = A.arrays()
    before = oracle.get_threads()
    cb = bench.cpu_baseline(rp, c, v, b, S.sum_dof(), argparse.Namespace(n=3, p=4, cpu_sample_iters=2), 30)
    assert oracle.get_threads() == before
    assert cb["kind"] == "port" and cb["cores"] == before and cb["value"] > 0
    assert cb["single_core"]["cores"] == 1 and cb["single_core"]["value"] > 0
