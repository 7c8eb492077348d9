"""Pins the numpy restatement of the operators to the reference's own OpenCL
kernels compiled for the host (oracle/refkernels).  Runs where the reference
sources are available; FP32 kernels against the FP32 restatement."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import nesta_ref as R
from oracle import refkernels as K
from tests.conftest import rel_l2

if K.build() is None or not K.available():
    pytest.skip("reference kernel sources not available", allow_module_level=True)


def _rand(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize("W,H,F,C", [(8, 8, 2, 1), (16, 24, 3, 2), (40, 32, 5, 4)])
def test_operators_match_reference_kernels(W, H, F, C):
    rng = np.random.default_rng(W + 10 * F + C)
    x, k, S = _rand(rng, (F, H, W)), _rand(rng, (F, C, H, W)), _rand(rng, (C, H, W))
    mask = ((rng.random((F, H, W)) > 0.5) * 255).astype(np.uint8)
    assert np.array_equal(K.ttv(x, True), R.ttv(x, True))
    assert np.array_equal(K.ttv(x, False), R.ttv(x, False))
    assert rel_l2(K.normalize(x, 0.6), R.normalize(x.astype(np.complex128), 0.6)) < 1e-6
    assert rel_l2(K.sensmul(x, S, False), R.sensmul(x.astype(np.complex128), S.astype(np.complex128), False)) < 1e-6
    assert rel_l2(K.sensmul(k, S, True), R.sensmul(k.astype(np.complex128), S.astype(np.complex128), True)) < 1e-6
    assert rel_l2(K.coilsum(k), R.coilsum(k.astype(np.complex128))) < 1e-6
    assert np.array_equal(K.apply_mask(k, mask), R.apply_mask(k, mask))
    assert rel_l2(K.abs2(k), R.complex_abs2(k.astype(np.complex128))) < 1e-6
    assert rel_l2(K.cabs(x), R.complex_abs(x.astype(np.complex128))) < 1e-6
    # RSoS: the FP32 restatement follows the kernel's accumulation order exactly
    assert np.array_equal(K.rss(k), R.rss(k))


def test_ttv_edge_frames_follow_reference_kernel():
    """temporalTV.cl: frame 0 of the forward difference wraps to frame F-1 and
    the adjoint's last frame wraps to frame 0."""
    x = np.arange(3 * 8 * 8, dtype=np.float32).reshape(3, 8, 8).astype(np.complex64)
    fwd = K.ttv(x, True)
    adj = K.ttv(x, False)
    assert np.array_equal(fwd[0], x[0] - x[2]) and np.array_equal(adj[2], x[0] - x[2])
