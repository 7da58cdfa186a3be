"""Device-side error paths, made to fire without any GPU fault.

* Traversal stack overflow: with RTX_OPT_STACK_LIMIT lowered to 2 entries,
  rays that need more stop in bounds and set the context's error word; every
  traversing call (render, per-path trace, primary hits, AOVs, arbitrary rays)
  returns RTX_ERR_DEVICE "traversal stack overflow".  With the limit restored
  the same context renders bit-identically to before.
* Bounded tensor-core barrier wait: a barrier that nothing arrives on, waited
  on with the tensor-core kernels' bounded wait and a short bound, reports
  "tensor-core barrier wait timed out"; the context stays usable.
"""
import numpy as np
import pytest

from helpers import same_bits
from rendertoy_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_stack_overflow_is_reported_and_recoverable(ctx):
    import rendertoy_gb300 as rt
    sc = scenes.displaced_icosphere(subdiv=4)
    ctx.upload(sc)
    W, H = 48, 32
    clean = ctx.render_pt(W, H, 2, 8, seed=1)
    assert ctx.get_option(rt.OPT_STACK_LIMIT) == 64
    calls = {
        "render_pt": lambda: ctx.render_pt(W, H, 2, 8, seed=1),
        "trace_paths": lambda: ctx.trace_paths(W, H, 0, 1, 8, seed=1),
        "primary": lambda: ctx.primary(W, H),
        "aov": lambda: ctx.aov(W, H, 700.0, 1500.0),
    }
    try:
        for trav in (2, 0):  # the 4-wide tree (default) and the binary tree
            ctx.set_option(rt.OPT_TRAVERSAL, trav)
            ctx.set_option(rt.OPT_STACK_LIMIT, 2)
            for name, fn in calls.items():
                with pytest.raises(rt.RtxError) as ei:
                    fn()
                assert ei.value.code == 5, (trav, name, ei.value)  # RTX_ERR_DEVICE
                assert "traversal stack overflow" in str(ei.value), (trav, name, ei.value)
            ctx.set_option(rt.OPT_STACK_LIMIT, 64)
    finally:
        ctx.set_option(rt.OPT_STACK_LIMIT, 64)
        ctx.set_option(rt.OPT_TRAVERSAL, 2)
    again = ctx.render_pt(W, H, 2, 8, seed=1)
    assert same_bits(clean, again)
    with pytest.raises(rt.RtxError):
        ctx.set_option(rt.OPT_STACK_LIMIT, 65)


def test_bounded_barrier_wait_reports_timeout(ctx):
    for polls in (1, 256):
        r = ctx.L.rtx_selftest_wait_timeout(ctx.h, polls)
        assert r == 5, r  # RTX_ERR_DEVICE
        assert b"tensor-core barrier wait timed out" in ctx.L.rtx_last_error(ctx.h)
    # the context still works: a tensor-core GEMM right after
    rng = np.random.RandomState(0)
    a16 = (rng.normal(size=(128, 64)).astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)
    b16 = (rng.normal(size=(64, 64)).astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)
    widen = lambda x: (x.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    C = ctx.gemm_bf16(a16, b16)
    assert np.allclose(C, widen(a16) @ widen(b16).T, rtol=1e-4, atol=1e-3)
