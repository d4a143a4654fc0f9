"""The allocation-free matrix-free apply (tsem_mf_apply_device_noalloc) through the
C ABI.  It serves callers that may not allocate device memory while they run (a
host that hands all device memory to its own pool, a serving loop that must not
stall on an allocator).  On every level of the hierarchy, the assembled coarse
levels included, it agrees with tsem_mf_apply_device on two calls in a row and
leaves the device's free memory unchanged; it rejects a level whose scratch does
not fit its static array, and an output that overlaps the input.  Collected last
so that it also runs after every other test."""
import ctypes

import numpy as np
import pytest

from tsemlib_gb300 import _lib, mesh, tsem

pytestmark = pytest.mark.gpu

# FP32 arithmetic on both sides: the allocation-free call runs the CUDA-core GEMM and an
# atomic scatter on every level, tsem_mf_apply_device the tensor-core GEMMs (split TF32)
# and, on the coarse levels, the assembled FP32 CSR matrix
TOL = 1e-6


def _solver(n, p, shuffle=True):
    m = mesh.kuhn_cube(n, 0.1, 1)
    if shuffle:
        m = mesh.shuffle_local_order(m, 1)
    m = mesh.mark_box_boundary(m, [(0, 0.0), (0, 1.0)])
    T = tsem.TSEM(p, 4, m)
    A = T.stiff_matrix.copy()
    T.impose_zero_boundary_condition(A, None, 1)
    return tsem.MixedSolver(T, A, 1, order_step=2, smooth=2)


def _noalloc(mx, level, x, y, stream):
    return _lib.lib().tsem_mf_apply_device_noalloc(mx._h.h, level, _lib.ptr(x.data_ptr()), _lib.ptr(y.data_ptr()),
                                                   _lib.stream_ptr(stream.cuda_stream))


@pytest.mark.parametrize("n,p", [(3, 6), (2, 5)])
def test_noalloc_apply_matches_apply(n, p):
    import torch
    mx = _solver(n, p)
    s = torch.cuda.Stream()
    g = torch.Generator(device="cuda").manual_seed(3)
    for level in range(mx.num_levels):
        size = mx.level_size(level)
        x = torch.randn(size, device="cuda", dtype=torch.float32, generator=g)
        y_ref = torch.empty_like(x)
        y1 = torch.full_like(x, 7.0)        # the call overwrites y entirely
        y2 = torch.full_like(x, -3.0)
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            mx.apply_device(level, x.data_ptr(), y_ref.data_ptr(), s.cuda_stream)
        assert _noalloc(mx, level, x, y1, s) == 0, _lib.lib().tsem_last_error()
        s.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        assert _noalloc(mx, level, x, y1, s) == 0, _lib.lib().tsem_last_error()
        assert _noalloc(mx, level, x, y2, s) == 0, _lib.lib().tsem_last_error()
        s.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        scale = torch.linalg.norm(y_ref).item()
        assert scale > 0 and torch.isfinite(y_ref).all()
        for y in (y1, y2):
            assert torch.linalg.norm(y - y_ref).item() <= TOL * scale, level


def test_noalloc_apply_rejects_oversized_level():
    import torch
    # N = 18, p = 6: the fine level needs 4 * (64 + 2 * 35072 * 84) bytes > 16 MiB,
    # level 1 (p = 4, 35 local modes) fits
    mx = _solver(18, 6, shuffle=False)
    s = torch.cuda.Stream()
    x = torch.ones(mx.level_size(0), device="cuda", dtype=torch.float32)
    y = torch.zeros_like(x)
    rc = _noalloc(mx, 0, x, y, s)
    assert rc == 6, rc      # TSEM_INVALID
    msg = _lib.lib().tsem_last_error()
    msg = msg.decode() if isinstance(msg, bytes) else str(msg)
    assert "at most" in msg and str(16 << 20) in msg
    x1 = torch.ones(mx.level_size(1), device="cuda", dtype=torch.float32)
    y1 = torch.empty_like(x1)
    y_ref = torch.empty_like(x1)
    with torch.cuda.stream(s):
        mx.apply_device(1, x1.data_ptr(), y_ref.data_ptr(), s.cuda_stream)
    assert _noalloc(mx, 1, x1, y1, s) == 0
    s.synchronize()
    assert torch.linalg.norm(y1 - y_ref).item() <= TOL * torch.linalg.norm(y_ref).item()


def test_noalloc_apply_rejects_overlapping_vectors():
    import torch
    mx = _solver(2, 4)
    s = torch.cuda.Stream()
    n = mx.level_size(0)
    buf = torch.ones(2 * n, device="cuda", dtype=torch.float32)
    x = buf[:n]
    assert _noalloc(mx, 0, x, x, s) == 6             # y == x
    assert _noalloc(mx, 0, x, buf[n // 2:], s) == 6  # partial overlap
    y = buf[n:]
    assert _noalloc(mx, 0, x, y, s) == 0, _lib.lib().tsem_last_error()
    s.synchronize()
    assert torch.isfinite(y).all()
