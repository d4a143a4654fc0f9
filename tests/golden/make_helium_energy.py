"""Generate the oracle's self-consistent helium energy on a small graded mesh.

tests/ks_oracle.py runs the Kohn-Sham loop of tsemlib_gb300.ks (exchange-only LDA,
multipole Hartree boundary data) on the CPU oracle in FP64.  Here it runs once on
the Kuhn mesh graded towards the nucleus with 2 geometric steps per half-axis
(ratio 1.15, half-width 10), p = 4, quadrature q = 6, and the converged energy and
lowest eigenvalues are kept:

  helium_graded2_p4.npz   energy, eigenvalues[4], SCF iterations, mesh parameters

    python tests/golden/make_helium_energy.py

The GPU test (tests/test_gpu_ks.py) runs ks.helium on the same mesh and compares.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests import ks_oracle  # noqa: E402
from tsemlib_gb300 import mesh  # noqa: E402

N_HALF, RATIO, HALF_WIDTH, P = 2, 1.15, 10.0, 4


def main():
    coords = mesh.graded_coords(N_HALF, RATIO, HALF_WIDTH)
    m = mesh.kuhn_cube(len(coords) - 1, 0.0, 0, coords=coords)
    t = time.time()
    E, lam, it = ks_oracle.helium(m, P, tol=1e-10)
    print(f"E = {E!r}  eigenvalues {lam}  {it} SCF iterations  {time.time() - t:.1f} s")
    np.savez(os.path.join(HERE, "helium_graded2_p4.npz"), energy=E, eigenvalues=np.asarray(lam), iterations=it,
             n_half=N_HALF, ratio=RATIO, half_width=HALF_WIDTH, p=P)


if __name__ == "__main__":
    main()
