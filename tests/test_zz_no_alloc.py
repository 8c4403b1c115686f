"""The allocation-free triangle count (xgm_tc_solver_static), called through the C ABI.

Callers that cannot allocate device memory while they count (a host framework that owns
all device memory through its own allocator, a hot loop with no room for cudaMalloc)
use this entry point; its scratch is a fixed file-scope device array.  It must give the
same count as the allocating xgm_tc_solver, call after call (the array keeps the
previous call's contents, so every call has to reset what it reuses), and once a
device is set up its calls must not change the device's free memory.  Collected last on
purpose.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_tc(xgm, ctx, g) -> int:
    out = ctypes.c_uint64()
    st = xgm.lib().xgm_tc_solver_static(ctx._h, g._h, ctypes.byref(out))
    xgm._check(st, ctx)
    return int(out.value)


def _tc(xgm, ctx, g) -> int:
    out = ctypes.c_uint64()
    xgm._check(xgm.lib().xgm_tc_solver(ctx._h, g._h, ctypes.byref(out)), ctx)
    return int(out.value)


def test_static_scratch_triangle_count_matches(xgm):
    ctx = xgm.Context(0)
    try:
        # an R-MAT graph (warp and CTA tasks) and a complete graph whose lowest-ranked
        # vertices have out-degree > 1024 (hub sub-tasks)
        nv, s, d = xgm.gen_rmat(16, 16, seed=1)
        g1 = ctx.graph_from_edges(nv, s, d)
        n = 1400
        iu = np.triu_indices(n, 1)
        g2 = ctx.graph_from_edges(n, iu[0].astype(np.int32), iu[1].astype(np.int32))
        for g in (g1, g2, g1):
            want = _tc(xgm, ctx, g)
            assert _static_tc(xgm, ctx, g) == want
            assert _static_tc(xgm, ctx, g) == want  # second call in a row, same array
        # beyond the array's capacity: a clear error, not a wrong count
        big = ctx.graph_from_edges((1 << 21) + 1, np.array([0], np.int32), np.array([1], np.int32))
        with pytest.raises(xgm.XgmError) as e:
            _static_tc(xgm, ctx, big)
        assert e.value.status == xgm.ERR_UNSUPPORTED
    finally:
        ctx.close()


def test_static_calls_leave_free_memory_unchanged(xgm):
    torch = pytest.importorskip("torch")
    ctx = xgm.Context(0)
    try:
        nv, s, d = xgm.gen_rmat(14, 16, seed=3)
        g = ctx.graph_from_edges(nv, s, d)
        want = _tc(xgm, ctx, g)
        assert _static_tc(xgm, ctx, g) == want  # first call on the device: set-up
        free0, _ = torch.cuda.mem_get_info(0)
        got = [_static_tc(xgm, ctx, g) for _ in range(3)]
        free1, _ = torch.cuda.mem_get_info(0)
        assert got == [want] * 3
        assert free1 == free0, f"device free memory moved by {free0 - free1} bytes"
        # a graph owned by another context is refused, not counted
        other = xgm.Context(0)
        try:
            g_other = other.graph_from_edges(nv, s, d)
            with pytest.raises(xgm.XgmError) as e:
                _static_tc(xgm, ctx, g_other)
            assert e.value.status == xgm.ERR_INVALID
            g_other.close()
        finally:
            other.close()
    finally:
        ctx.close()
