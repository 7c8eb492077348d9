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

import ctypes

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


def _device_free_bytes() -> int:
    """cudaMemGetInfo's free bytes, from the CUDA runtime the library loaded."""
    g.lib()
    with open("/proc/self/maps") as fh:
        paths = sorted({ln.split()[-1] for ln in fh if "libcudart.so" in ln})
    assert paths, "libcudart not loaded"
    rt = ctypes.CDLL(paths[0])
    free, total = ctypes.c_size_t(0), ctypes.c_size_t(0)
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_static_entry_point_allocates_nothing(built_lib):
    # a context of its own: nothing else grows device memory between the calls
    W, H, F, C = 64, 64, 2, 4
    p = synth.make_fully_sampled(W, H, C, seed=5)
    y = np.ascontiguousarray(np.repeat(p.y, F, axis=0))
    with g.Context(0) as c:
        dy, dS = c.to_device(y), c.to_device(p.S)
        out = c.zeros((F, H, W), np.complex64)
        _abi.call("gbn_simple_recon_static", c.handle, dy.ptr, dS.ptr, out.ptr, W, H, F, C)  # loads its kernels
        c.sync()
        before = _device_free_bytes()
        for _ in range(3):
            _abi.call("gbn_simple_recon_static", c.handle, dy.ptr, dS.ptr, out.ptr, W, H, F, C)
        c.sync()
        assert _device_free_bytes() == before
        assert np.isfinite(out.get()).all()


@pytest.mark.parametrize("W,H,F,C", [
    (512, 512, 1, 8),   # F*H*C*W = 2^21 > 2^20
    (8, 512, 17, 1),    # F*H = 8704 > 8192 with F*H*C*W = 69632 within its limit
])
def test_static_scratch_rejects_oversized_problem(ctx, W, H, F, C):
    dy = ctx.zeros((F, C, H, W), np.complex64)
    dS = ctx.zeros((C, H, W), np.complex64)
    out = ctx.zeros((F, H, W), np.complex64)
    with pytest.raises(g.GbnError) as ei:
        _abi.call("gbn_simple_recon_static", ctx.handle, dy.ptr, dS.ptr, out.ptr, W, H, F, C)
    assert ei.value.code == _abi.GBN_ERR_UNSUPPORTED
    assert "static scratch" in str(ei.value)


def test_static_entry_point_reports_unsupported_length(ctx):
    dy = ctx.zeros((1, 1, 88, 8), np.complex64)  # 88 = 8 * 11 is not 7-smooth
    dS = ctx.zeros((1, 88, 8), np.complex64)
    out = ctx.zeros((1, 88, 8), np.complex64)
    with pytest.raises(g.GbnError) as ei:
        _abi.call("gbn_simple_recon_static", ctx.handle, dy.ptr, dS.ptr, out.ptr, 8, 88, 1, 1)
    assert ei.value.code == _abi.GBN_ERR_UNSUPPORTED
    assert "W=8, H=88" in str(ei.value)
