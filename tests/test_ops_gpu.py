"""Per-operator parity on the GPU through the C ABI against the CPU oracle
(FP64 evaluation of the same operator): relative L2 <= 1e-5, the per-operator
bar for the plain FP32 path."""
from __future__ import annotations

import numpy as np
import pytest

import opencliper_gb300 as g
from opencliper_gb300 import api
from oracle import nesta_ref as R
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5

SHAPES = [(8, 8, 2, 1), (16, 24, 3, 2), (32, 32, 4, 3), (40, 56, 2, 2), (64, 48, 5, 2), (96, 72, 2, 3),
          (120, 112, 2, 2), (128, 128, 3, 2), (144, 160, 2, 2), (168, 192, 2, 2), (200, 216, 1, 2),
          (224, 240, 2, 1), (256, 256, 3, 2), (280, 288, 1, 2), (320, 336, 1, 2), (360, 384, 1, 1),
          (392, 400, 1, 1), (432, 448, 1, 1), (480, 504, 1, 1), (512, 512, 1, 1), (384, 320, 2, 2)]


def _rand(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def _c128(a):
    return a.astype(np.complex128)


@pytest.mark.parametrize("W,H,F,C", SHAPES)
def test_fft2_and_encode_operators(ctx, W, H, F, C):
    rng = np.random.default_rng(W * 1000 + H)
    x, k, S = _rand(rng, (F, H, W)), _rand(rng, (F, C, H, W)), _rand(rng, (C, H, W))
    mask = ((rng.random((F, H, W)) > 0.5) * 255).astype(np.uint8)
    dx, dk, dS, dm = ctx.to_device(x), ctx.to_device(k), ctx.to_device(S), ctx.to_device(mask)
    ok = ctx.empty(k.shape, np.complex64)
    ox = ctx.empty(x.shape, np.complex64)
    api.op_fft2(ctx, -1, dk, ok)
    assert rel_l2(ok.get(), np.fft.fft2(_c128(k))) < TOL
    api.op_fft2(ctx, 1, dk, ok)
    assert rel_l2(ok.get(), np.fft.ifft2(_c128(k))) < TOL
    api.op_encode(ctx, dx, dS, dm, ok)
    assert rel_l2(ok.get(), R.encode(_c128(x), _c128(S), mask)) < TOL
    api.op_encode_adjoint(ctx, dk, dS, ox)
    assert rel_l2(ox.get(), R.encode_adjoint(_c128(k), _c128(S))) < TOL
    api.simple_recon(ctx, dk, dS, ox)
    assert rel_l2(ox.get(), R.simple_recon(_c128(k), _c128(S))) < TOL


def test_simple_recon_repeated_calls(ctx):
    """A repeated call with the same shape and buffers reuses the tables the
    first call left in the context's scratch (2 launches instead of 5); new
    data in the same buffers, another operator using the scratch in between,
    and another shape all give the oracle's result."""
    rng = np.random.default_rng(11)
    W, H, F, C = 64, 48, 2, 3
    k1, k2, S = _rand(rng, (F, C, H, W)), _rand(rng, (F, C, H, W)), _rand(rng, (C, H, W))
    dk, dS = ctx.to_device(k1), ctx.to_device(S)
    ox = ctx.empty((F, H, W), np.complex64)
    counts = []
    for k in (k1, k2, k2):
        dk.set(k)
        n0 = ctx.launch_count()
        api.simple_recon(ctx, dk, dS, ox)
        counts.append(ctx.launch_count() - n0)
        assert rel_l2(ox.get(), R.simple_recon(_c128(k), _c128(S))) < TOL
    assert counts[1] < counts[0] and counts[2] == counts[1]
    api.op_encode_adjoint(ctx, dk, dS, ox)  # another user of the scratch
    n0 = ctx.launch_count()
    api.simple_recon(ctx, dk, dS, ox)
    assert ctx.launch_count() - n0 == counts[0]
    assert rel_l2(ox.get(), R.simple_recon(_c128(k2), _c128(S))) < TOL
    k3, S3 = _rand(rng, (1, 2, 40, 32)), _rand(rng, (2, 40, 32))
    ox3 = ctx.empty((1, 40, 32), np.complex64)
    api.simple_recon(ctx, ctx.to_device(k3), ctx.to_device(S3), ox3)
    assert rel_l2(ox3.get(), R.simple_recon(_c128(k3), _c128(S3))) < TOL


def test_fft2_in_place(ctx):
    rng = np.random.default_rng(0)
    k = _rand(rng, (3, 2, 48, 40))
    d = ctx.to_device(k)
    api.op_fft2(ctx, -1, d, d)
    assert rel_l2(d.get(), np.fft.fft2(_c128(k))) < TOL


@pytest.mark.parametrize("W,H,F,C", [(8, 8, 2, 1), (24, 16, 3, 2), (64, 48, 7, 3), (256, 256, 20, 12)])
def test_pointwise_operators(ctx, W, H, F, C):
    rng = np.random.default_rng(F * 31 + C)
    x, k, S = _rand(rng, (F, H, W)), _rand(rng, (F, C, H, W)), _rand(rng, (C, H, W))
    mask = ((rng.random((F, H, W)) > 0.5) * 255).astype(np.uint8)
    dx, dk, dS, dm = ctx.to_device(x), ctx.to_device(k), ctx.to_device(S), ctx.to_device(mask)
    ox, ok = ctx.empty(x.shape, np.complex64), ctx.empty(k.shape, np.complex64)
    api.op_ttv(ctx, 1, dx, ox)
    assert rel_l2(ox.get(), R.ttv(_c128(x), True)) < TOL
    api.op_ttv(ctx, 0, dx, ox)
    assert rel_l2(ox.get(), R.ttv(_c128(x), False)) < TOL
    api.op_normalize(ctx, dx, ox, 0.7)
    assert rel_l2(ox.get(), R.normalize(_c128(x), 0.7)) < TOL
    api.op_sensmul(ctx, False, dx, dS, ok)
    assert rel_l2(ok.get(), R.sensmul(_c128(x), _c128(S), False)) < TOL
    api.op_sensmul(ctx, True, dk, dS, ok)
    assert rel_l2(ok.get(), R.sensmul(_c128(k), _c128(S), True)) < TOL
    api.op_coilsum(ctx, dk, ox)
    assert rel_l2(ox.get(), R.coilsum(_c128(k))) < TOL
    dk2 = ctx.to_device(k)
    api.op_mask(ctx, dk2, dm)
    assert np.array_equal(dk2.get(), R.apply_mask(k, mask))
    api.op_abs(ctx, dx, ox)
    assert rel_l2(ox.get(), R.complex_abs(_c128(x))) < TOL
    api.op_abs(ctx, dx, ox, squared=True)
    assert rel_l2(ox.get(), R.complex_abs2(_c128(x))) < TOL


def test_normalize_in_place_and_small_values(ctx):
    x = np.array([[[1e-6 + 1e-6j, 3 + 4j, 0j, -2e-3 + 0j] * 2]], np.complex64)
    d = ctx.to_device(x)
    api.op_normalize(ctx, d, d, 1e-3)
    assert rel_l2(d.get(), R.normalize(_c128(x), 1e-3)) < TOL


def test_rowmask_expansion(ctx):
    rng = np.random.default_rng(3)
    rm = (rng.random((4, 24)) > 0.5).astype(np.uint32)
    drm = ctx.to_device(rm)
    pm = ctx.empty((4, 24, 16), np.uint8)
    api.op_rowmask_to_pixelmask(ctx, drm, pm)
    assert np.array_equal(pm.get(), R.rowmask_to_pixelmask(rm, 16))
    bad = rm.copy()
    bad[1, 3] = 2
    with pytest.raises(g.GbnError) as ei:
        api.op_rowmask_to_pixelmask(ctx, ctx.to_device(bad), pm)
    assert ei.value.code == -1


def test_adjoint_identity_on_gpu(ctx):
    rng = np.random.default_rng(4)
    F, C, H, W = 3, 4, 40, 48
    x, k, S = _rand(rng, (F, H, W)), _rand(rng, (F, C, H, W)), _rand(rng, (C, H, W))
    mask = ((rng.random((F, H, W)) > 0.5) * 255).astype(np.uint8)
    dm = ctx.to_device(mask)
    Ex = ctx.empty(k.shape, np.complex64)
    api.op_encode(ctx, ctx.to_device(x), ctx.to_device(S), dm, Ex)
    km = ctx.to_device(k)
    api.op_mask(ctx, km, dm)
    EHk = ctx.empty(x.shape, np.complex64)
    api.op_encode_adjoint(ctx, km, ctx.to_device(S), EHk)
    lhs = np.vdot(_c128(Ex.get()), _c128(k))
    rhs = np.vdot(_c128(x), _c128(EHk.get()))
    assert abs(lhs - rhs) < 1e-5 * abs(lhs)


def test_errors_are_reported(ctx):
    rng = np.random.default_rng(5)
    k = ctx.to_device(_rand(rng, (1, 1, 8, 11 * 8)))  # W = 88 = 8*11 is not 7-smooth
    with pytest.raises(g.GbnError) as ei:
        api.op_fft2(ctx, -1, k, k)
    assert ei.value.code == -2
    x = ctx.to_device(_rand(rng, (2, 8, 12)))  # width not a multiple of 8
    with pytest.raises(g.GbnError) as ei:
        api.op_ttv(ctx, 1, x, ctx.empty((2, 8, 12), np.complex64))
    assert ei.value.code == -1
    with pytest.raises(g.GbnError):
        api.op_fft2(ctx, 7, k, k)


def test_operators_match_reference_kernel_outputs(ctx):
    """GPU operators against outputs of the reference's own OpenCL kernels
    compiled for the host (tests/golden/ops_refkernels.npz)."""
    import os
    from tests.conftest import ROOT
    d = np.load(os.path.join(ROOT, "tests", "golden", "ops_refkernels.npz"))
    x, k, S, mask = d["x"], d["k"], d["S"], d["mask"]
    F, C, H, W = k.shape
    dx, dk, dS, dm = ctx.to_device(x), ctx.to_device(k), ctx.to_device(S), ctx.to_device(mask)
    ox, ok = ctx.empty(x.shape, np.complex64), ctx.empty(k.shape, np.complex64)
    api.op_ttv(ctx, 1, dx, ox)
    assert np.array_equal(ox.get(), d["ttv_fwd"])
    api.op_ttv(ctx, 0, dx, ox)
    assert np.array_equal(ox.get(), d["ttv_adj"])
    api.op_normalize(ctx, dx, ox, float(d["mu"]))
    assert rel_l2(ox.get(), d["normalize"]) < TOL
    api.op_sensmul(ctx, False, dx, dS, ok)
    assert rel_l2(ok.get(), d["sensmul_x"]) < TOL
    api.op_sensmul(ctx, True, dk, dS, ok)
    assert rel_l2(ok.get(), d["sensmul_k_conj"]) < TOL
    api.op_coilsum(ctx, dk, ox)
    assert rel_l2(ox.get(), d["coilsum"]) < TOL
    dk2 = ctx.to_device(k)
    api.op_mask(ctx, dk2, dm)
    assert np.array_equal(dk2.get(), d["mask_k"])
    api.op_abs(ctx, dk, ok, squared=True)
    assert rel_l2(ok.get(), d["abs2"]) < TOL
    api.op_abs(ctx, dx, ox)
    assert rel_l2(ox.get(), d["abs"]) < TOL
    api.op_rss(ctx, dk, ox)
    assert rel_l2(ox.get(), d["rss"]) < TOL


@pytest.mark.parametrize("W,H,F,C", [(32, 32, 1, 8), (48, 40, 3, 5), (256, 256, 1, 8)])
def test_simple_recon_sos(ctx, W, H, F, C):
    """SimpleMRIReconSOS: inverse FFT per coil, root sum of squares; input untouched."""
    rng = np.random.default_rng(W + C)
    y = _rand(rng, (F, C, H, W))
    dy, ox = ctx.to_device(y), ctx.empty((F, H, W), np.complex64)
    api.simple_recon_sos(ctx, dy, ox)
    ref = R.simple_recon_sos(_c128(y))
    out = ox.get()
    assert rel_l2(out, ref) < TOL
    assert not out.imag.any()
    assert np.array_equal(dy.get(), y)
