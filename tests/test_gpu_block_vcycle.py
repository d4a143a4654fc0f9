"""Block V-cycles of the mixed solver: a block of columns runs as one V-cycle whose
launches cover all columns (the fused-gather element GEMM over (column, tile)
pairs, the scatters and coarse sweeps over blockIdx.y); every column must come out
bit for bit as a one-column V-cycle of the same vector."""
import numpy as np
import pytest

from tests.test_gpu_parity import _cfg1
from tsemlib_gb300 import tsem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,p,shuffle,ncol", [(3, 6, False, 5), (3, 5, True, 3), (2, 4, False, 1)])
def test_block_vcycle_equals_column_vcycles(n, p, shuffle, ncol):
    torch = pytest.importorskip("torch")
    m = _cfg1(n, p, shuffle)
    T = tsem.TSEM(p, p + 2, m)
    A = T.stiff_matrix.copy()
    T.impose_zero_boundary_condition(A, None, 1)
    mx = tsem.MixedSolver(T, A, 1, order_step=2)
    nd = T.n_dof_total
    g = torch.Generator(device="cpu").manual_seed(11)
    r = torch.randn(ncol, nd, generator=g).float().cuda()
    zb = torch.empty_like(r)
    mx.vcycle_device(ncol, r.data_ptr(), zb.data_ptr())
    torch.cuda.synchronize()
    for j in range(ncol):
        rj = r[j].clone()
        zj = torch.empty_like(rj)
        mx.vcycle_device(1, rj.data_ptr(), zj.data_ptr())
        torch.cuda.synchronize()
        assert torch.equal(zj, zb[j]), j
    # a preconditioner: z is finite, nonzero, and positively correlated with r
    assert torch.isfinite(zb).all()
    for j in range(ncol):
        assert float((zb[j] * r[j]).sum()) > 0.0
