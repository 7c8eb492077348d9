"""Allocation-free SimpleMRIRecon (gbn_simple_recon_static).

Callers that cannot allocate device memory at reconstruction time -- code
running while a stream is captured into a CUDA graph, or hosts that own all
device memory in fixed pools -- use this entry point: its working memory is a
fixed array inside the library instead of a cudaMalloc.  The test calls it
through the C ABI twice in a row (the second call reuses the scratch left by
the first) and checks both results against the allocating entry point
gbn_simple_recon, then checks that oversized problems are refused.
"""
from __future__ import annotations

import numpy as np
import pytest

import opencliper_gb300 as g
from opencliper_gb300 import _abi, api, synth
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the per-operator bar used by the other GPU operator tests


@pytest.mark.parametrize("W,H,F,C", [(256, 256, 1, 8), (48, 40, 3, 4)])
def test_static_scratch_matches_allocating_entry_point(ctx, W, H, F, C):
    p = synth.make_fully_sampled(W, H, C, seed=31)
    y = np.repeat(p.y, F, axis=0) if F > 1 else p.y
    y = np.ascontiguousarray(y * (1 + 0.1 * np.arange(F)[:, None, None, None]).astype(np.complex64))
    dy, dS = ctx.to_device(y), ctx.to_device(p.S)
    ref = ctx.empty((F, H, W), np.complex64)
    api.simple_recon(ctx, dy, dS, ref)
    want = ref.get()
    for _ in range(2):
        out = ctx.zeros((F, H, W), np.complex64)
        _abi.call("gbn_simple_recon_static", ctx.handle, dy.ptr, dS.ptr, out.ptr, W, H, F, C)
        got = out.get()
        assert np.isfinite(got).all()
        assert rel_l2(got, want) <= TOL


def test_static_scratch_rejects_oversized_problem(ctx):
    W = H = 512
    F, C = 1, 8  # F*H*C*W = 2^21 > 2^20
    dy = ctx.zeros((F, C, H, W), np.complex64)
    dS = ctx.zeros((C, H, W), np.complex64)
    out = ctx.zeros((F, H, W), np.complex64)
    with pytest.raises(g.GbnError) as ei:
        _abi.call("gbn_simple_recon_static", ctx.handle, dy.ptr, dS.ptr, out.ptr, W, H, F, C)
    assert ei.value.code == _abi.GBN_ERR_UNSUPPORTED
    assert "static scratch" in str(ei.value)
