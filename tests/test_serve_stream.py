"""The serving workload's request generator (serve.stream, CPU only): 2000 requests
from a Poisson process at the given rate, 80 % Poisson / 20 % eigen with k uniform
in 4..32, N uniform in 4..32, p uniform in 2..8, node jitter 0.1 h, tolerance 1e-10;
the same seed gives the same stream, and a sweep over rates keeps the requests and
rescales only their arrivals."""
import numpy as np

from tsemlib_gb300 import serve


def test_stream_follows_the_serving_distributions():
    rate = 100.0
    reqs = serve.stream(2000, rate, seed=2024)
    assert len(reqs) == 2000
    kinds = np.array([r["kind"] == "eigen" for r in reqs])
    # binomial(2000, 0.2): standard deviation about 18
    assert abs(kinds.sum() - 400) <= 90
    n = np.array([r["n"] for r in reqs])
    p = np.array([r["p"] for r in reqs])
    k = np.array([r["k"] for r in reqs])
    assert set(n.tolist()) == set(range(4, 33)) and set(p.tolist()) == set(range(2, 9))
    assert set(k[kinds].tolist()) <= set(range(4, 33)) and len(set(k[kinds].tolist())) >= 25
    assert np.all(k[~kinds] == 0)
    assert all(r["jitter"] == 0.1 and r["tol"] == 1e-10 for r in reqs)
    assert len({r["seed"] for r in reqs}) == 2000
    t = np.array([r["arrival"] for r in reqs])
    gaps = np.diff(np.r_[0.0, t])
    assert np.all(gaps > 0)
    # exponential gaps of mean 1 / rate: the mean within a few standard errors
    assert abs(gaps.mean() * rate - 1.0) <= 5 / np.sqrt(2000)
    assert abs(gaps.std() * rate - 1.0) <= 0.15


def test_stream_is_seeded_and_rates_rescale_arrivals_only():
    a = serve.stream(300, 50.0, seed=7, n_range=(4, 16), p_range=(2, 6))
    b = serve.stream(300, 50.0, seed=7, n_range=(4, 16), p_range=(2, 6))
    assert a == b
    c = serve.stream(300, 200.0, seed=7, n_range=(4, 16), p_range=(2, 6))
    for x, y in zip(a, c):
        assert {k: v for k, v in x.items() if k != "arrival"} == {k: v for k, v in y.items() if k != "arrival"}
        assert abs(y["arrival"] * 200.0 - x["arrival"] * 50.0) <= 1e-9 * max(1.0, x["arrival"] * 50.0)
    assert max(r["n"] for r in a) <= 16 and max(r["p"] for r in a) <= 6
