"""Failure detection of the tensor-core kernels: a bounded device wait that gives up.

Every mbarrier wait in the matrix-free kernels gives up after a poll limit and
records an error code that the host turns into TSEM_TIMEOUT.  The test lowers the
limit of the waits that may give up to one poll (tsem_debug_wait_limit), so that
the fused-gather BF16 and split-TF32 GEMMs give up on their first wait; the
waits a kernel makes for its own copies and MMAs before it exits keep their full
limit, so every kernel still exits cleanly.  The solve must come back with
TSEM_TIMEOUT, and the next solve on the same solver, with the default limit, must
succeed and give the same answer as before.  Nothing faults, traps or hangs: the
giving up is the kernels' designed error path."""
import numpy as np
import pytest

from tsemlib_gb300 import _lib, mesh, tsem
from tsemlib_gb300 import manufactured as mf

pytestmark = pytest.mark.gpu


def test_wait_timeout_is_reported_and_the_solver_recovers():
    m = mesh.mark_box_boundary(mesh.kuhn_cube(3, 0.1, 2), [(0, 0.0), (0, 1.0)])
    T = tsem.TSEM(6, 8, m)
    A = T.stiff_matrix.copy()
    b = T.calc_rhs(mf.f_cfg1)
    T.impose_neumann(b, mf.neumann_cfg1, 2)
    T.impose_boundary_condition(A, b, mf.u_cfg1, True, 1)
    mx = tsem.MixedSolver(T, A, 1, order_step=2, tol_rel=1e-10)
    x0 = np.zeros(T.n_dof_total)
    assert mx.solve(x0, b)["status"] == "OK"
    L = _lib.lib()
    assert L.tsem_debug_wait_limit(1) == 0
    try:
        x1 = np.zeros(T.n_dof_total)
        with pytest.raises(tsem.TsemError) as e:
            mx.solve(x1, b)
        assert e.value.status == 5, e.value          # TSEM_TIMEOUT
        assert "bounded wait" in str(e.value)
    finally:
        assert L.tsem_debug_wait_limit(0) == 0
    x2 = np.zeros(T.n_dof_total)
    st = mx.solve(x2, b)
    assert st["status"] == "OK" and st["residual_rel"] <= 1e-10
    assert np.abs(x2 - x0).max() <= 1e-9 * np.abs(x0).max()
