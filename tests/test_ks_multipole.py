"""Hartree boundary data of the Kohn-Sham loop: the density's multipole expansion
to quadrupole order (SCFIteration.cpp:70-153) against the exact Coulomb potential
of a cluster of point charges, evaluated far from it (CPU, numpy)."""
import numpy as np

from tsemlib_gb300 import ks


def test_multipole_expansion_matches_point_charges():
    rng = np.random.default_rng(11)
    pos = rng.uniform(-0.3, 0.3, (1, 40, 3))            # charge positions [1 element, 40 points, 3]
    w = rng.uniform(0.1, 1.0, (1, 40))                   # charges as weights, density 1
    c = ks.multipole_moments(w, pos, np.ones_like(w))
    assert abs(c[0] - w.sum()) <= 1e-12
    far = rng.normal(size=(500, 3))
    far *= (10.0 / np.linalg.norm(far, axis=-1))[:, None]
    exact = (w[0][None, :] / np.linalg.norm(far[:, None, :] - pos[0][None, :, :], axis=-1)).sum(axis=1)
    approx = ks.multipole_potential(c, far)
    # the first omitted term (octupole) is of relative size (a / r)^3 ~ 3e-5 here
    assert np.abs(approx - exact).max() <= 1e-4 * np.abs(exact).max()
    # and the expansion improves on the monopole term alone by orders of magnitude
    mono = c[0] / np.linalg.norm(far, axis=-1)
    assert np.abs(approx - exact).max() < 1e-2 * np.abs(mono - exact).max()
