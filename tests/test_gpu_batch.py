"""Batched solves (tsem_solve_batch, tsem_batch_*): systems of different meshes and
orders solved together, the same order's V-cycle steps as single launches over a
ragged table of all members' elements and DOFs.  Each system's result equals the one
it reaches alone to the solve tolerance (the same kernels per element and per DOF;
only the order of the atomically accumulated inner products differs), also when
members retire at different rounds and join again after their refinement steps."""
import ctypes

import numpy as np
import pytest

from tsemlib_gb300 import _lib, mesh, tsem
from tsemlib_gb300 import manufactured as mf

pytestmark = pytest.mark.gpu


def _system(n, p, seed):
    m = mesh.mark_box_boundary(mesh.kuhn_cube(n, 0.1, seed), [(0, 0.0), (0, 1.0)])
    T = tsem.TSEM(p, p + 2, m)
    A = T.stiff_matrix.copy()
    b = T.calc_rhs(mf.f_cfg1)
    T.impose_neumann(b, mf.neumann_cfg1, 2)
    T.impose_boundary_condition(A, b, mf.u_cfg1, True, 1)
    return T, A, b


def _alone(systems, solvers):
    out = []
    for (T, A, b), sv in zip(systems, solvers):
        x = np.zeros(T.n_dof_total)
        st = sv.solve(x, b)
        assert st["status"] == "OK", st
        out.append((x, st))
    return out


def test_batch_equals_alone():
    # orders 2 .. 6 on meshes of four sizes; two systems share order 6 and two order 4
    specs = [(3, 6, 1), (4, 6, 2), (2, 4, 3), (5, 4, 4), (3, 5, 5), (4, 3, 6), (2, 2, 7)]
    systems = [_system(*sp) for sp in specs]
    solvers = [tsem.MixedSolver(T, A, 1, order_step=2, tol_rel=1e-10) for T, A, _ in systems]
    alone = _alone(systems, solvers)
    xs = [np.zeros(T.n_dof_total) for T, _, _ in systems]
    stats = tsem.solve_batch(solvers, [b for _, _, b in systems], xs)
    for (x0, st0), x, st, (T, A, b) in zip(alone, xs, stats, systems):
        assert st["status"] == "OK", st
        assert st["residual_rel"] <= 1e-10
        assert abs(st["iterations"] - st0["iterations"]) <= 1 and st["outer"] == st0["outer"]
        # the same kernels; the atomically accumulated inner products sum in another
        # order, so the iterates part at rounding level and both stop at 1e-10
        assert np.abs(x - x0).max() <= 1e-9 * np.abs(x0).max()
        r = A.vmult(x) - b
        assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(b)


def test_batch_of_one_order_shares_launches():
    """Four systems of order 6 on different meshes: the batch launches far fewer
    kernels than the four solves alone (one group launch per V-cycle step)."""
    specs = [(3, 6, 11), (4, 6, 12), (3, 6, 13), (5, 6, 14)]
    systems = [_system(*sp) for sp in specs]
    solvers = [tsem.MixedSolver(T, A, 1, order_step=2, tol_rel=1e-10) for T, A, _ in systems]
    L = _lib.lib()
    k0 = L.tsem_kernel_launches()
    alone = _alone(systems, solvers)
    k1 = L.tsem_kernel_launches()
    xs = [np.zeros(T.n_dof_total) for T, _, _ in systems]
    stats = tsem.solve_batch(solvers, [b for _, _, b in systems], xs)
    k2 = L.tsem_kernel_launches()
    for (x0, _), x, st in zip(alone, xs, stats):
        assert st["status"] == "OK", st
        assert np.abs(x - x0).max() <= 1e-9 * np.abs(x0).max()
    assert (k2 - k1) < 0.6 * (k1 - k0), (k1 - k0, k2 - k1)


def test_continuous_batch_submit_poll_cancel():
    """tsem_batch_submit / poll / cancel on device arrays: systems join while others
    are in flight, a cancelled one comes back with TSEM_INVALID, the rest equal their
    solves alone."""
    torch = pytest.importorskip("torch")
    specs = [(3, 6, 21), (2, 4, 22), (4, 6, 23), (3, 5, 24)]
    systems = [_system(*sp) for sp in specs]
    solvers = [tsem.MixedSolver(T, A, 1, order_step=2, tol_rel=1e-10) for T, A, _ in systems]
    alone = _alone(systems, solvers)
    L = _lib.lib()
    bt = ctypes.c_void_p()
    _lib.check(L.tsem_batch_create(None, ctypes.byref(bt)))
    try:
        bd = [torch.from_numpy(b).cuda() for _, _, b in systems]
        xd = [torch.zeros_like(b) for b in bd]
        torch.cuda.synchronize()
        tickets = {}

        def submit(i):
            t = ctypes.c_int64()
            _lib.check(L.tsem_batch_submit(bt, solvers[i]._h.h, ctypes.c_void_p(bd[i].data_ptr()),
                                           ctypes.c_void_p(xd[i].data_ptr()), ctypes.byref(t)))
            tickets[t.value] = i
            return t.value

        submit(0)
        submit(1)
        cancelled = submit(3)
        _lib.check(L.tsem_batch_cancel(bt, ctypes.c_int64(cancelled)))
        got = {}
        ids = (ctypes.c_int64 * 8)()
        sts = (_lib.Stats * 8)()
        nd, nf = ctypes.c_int32(), ctypes.c_int32()
        late = False
        for _ in range(100000):
            _lib.check(L.tsem_batch_poll(bt, 8, ids, sts, ctypes.byref(nd), ctypes.byref(nf)))
            for j in range(nd.value):
                got[tickets[ids[j]]] = sts[j].as_dict()
            if not late:
                submit(2)       # joins while the first ones are in flight
                late = True
            if nf.value == 0 and len(got) == 4:
                break
        assert len(got) == 4
        assert got[3]["status"] == "INVALID"
        torch.cuda.synchronize()
        for i in (0, 1, 2):
            assert got[i]["status"] == "OK", got[i]
            x0 = alone[i][0]
            assert np.abs(xd[i].cpu().numpy() - x0).max() <= 1e-9 * np.abs(x0).max()
    finally:
        L.tsem_batch_destroy(bt)
