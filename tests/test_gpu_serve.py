"""Request service (tsem_serve): every request's result is the same alone and in a
mix of overlapping requests; the memory budget admits and refuses by footprint."""
import numpy as np
import pytest

from tsemlib_gb300 import serve

pytestmark = pytest.mark.gpu


def _mix():
    return [dict(kind="poisson", n=4, p=4, seed=11, tol=1e-10, arrival=0.0),
            dict(kind="eigen", n=3, p=3, k=4, seed=12, tol=1e-10, arrival=0.0),
            dict(kind="poisson", n=5, p=3, seed=13, tol=1e-10, arrival=0.01),
            dict(kind="poisson", n=3, p=5, seed=14, tol=1e-10, arrival=0.02),
            dict(kind="eigen", n=4, p=2, k=6, seed=15, tol=1e-10, arrival=0.03),
            dict(kind="poisson", n=6, p=2, seed=16, tol=1e-10, arrival=0.03)]


def test_results_equal_alone_and_in_the_mix():
    reqs = _mix()
    mixed = serve.serve(reqs, workers=4, realtime=True)
    assert all(r["status"] == "OK" for r in mixed), mixed
    assert all(r["residual"] <= 1e-10 for r, q in zip(mixed, reqs) if q["kind"] == "poisson")
    for i, q in enumerate(reqs):
        alone = serve.serve([q], workers=1, realtime=False)[0]
        m = mixed[i]
        assert alone["status"] == "OK" and alone["n_dof"] == m["n_dof"]
        if q["kind"] == "poisson":
            # the inner solves are FP32 and their reductions run in a launch-dependent order:
            # equal to the solve tolerance
            assert abs(alone["checksum"] - m["checksum"]) <= 1e-8 * np.sqrt(alone["norm2"] * m["n_dof"])
        else:
            assert alone["lambda0"] == pytest.approx(m["lambda0"], rel=1e-9)
            assert alone["lambda_last"] == pytest.approx(m["lambda_last"], rel=1e-9)


def test_solution_output_and_plain_form_agree():
    q = dict(kind="poisson", n=4, p=4, seed=21, tol=1e-11, arrival=0.0)
    outs = {0: np.zeros((4 * 4 + 1) ** 3)}
    r = serve.serve([q], workers=1, realtime=False, outputs=outs)[0]
    outp = {0: np.zeros_like(outs[0])}
    rp = serve.serve([q], workers=1, realtime=False, plain=True, outputs=outp)[0]
    assert r["status"] == "OK" and rp["status"] == "OK"
    assert np.abs(outs[0] - outp[0]).max() <= 1e-8 * np.abs(outp[0]).max()


def test_budget_refuses_oversized_and_serialises():
    reqs = [dict(kind="poisson", n=4, p=3, seed=31, arrival=0.0), dict(kind="poisson", n=4, p=3, seed=32, arrival=0.0)]
    # a budget below one request's footprint: it runs alone and is refused
    r = serve.serve(reqs[:1], workers=2, realtime=False, budget_gb=1e-3)
    assert r[0]["status"] == "OOM_REFUSED"
    # a budget for one request at a time: the second starts after the first retires
    r = serve.serve(reqs, workers=2, realtime=False, budget_gb=0.09)
    assert all(x["status"] == "OK" for x in r)
    first, second = sorted(r, key=lambda x: x["finish_s"])
    assert second["queued_s"] >= first["finish_s"] - 1e-3
