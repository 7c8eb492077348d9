"""Motion-compensation oracle (oracle/motion.py) against the reference's own
interpolator / adjointInterpolator / initZeroRect / copyDataGPU kernels
compiled for the host, and the adjoint identity of the pair."""
from __future__ import annotations

import numpy as np
import pytest

from opencliper_gb300 import synth
from oracle import motion as M
from oracle import refkernels as K

_needs_ref = pytest.mark.skipif(K.build() is None, reason="reference kernel sources not available")


@_needs_ref
@pytest.mark.parametrize("W,H,F,seed", [(48, 40, 3, 1), (96, 80, 2, 2), (40, 160, 4, 3)])
def test_motion_oracle_matches_reference_kernels(W, H, F, seed):
    xn, xm, bb = synth.make_motion(W, H, F, seed=seed)
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal((F, H, W)) + 1j * rng.standard_normal((F, H, W))).astype(np.complex64)
    assert np.array_equal(K.mc(x, xn, xm, bb), M.warp(x, xn, xm, bb))
    assert np.array_equal(K.mc_adjoint(x, xn, xm, bb), M.warp_adjoint(x, xn, xm, bb))


def test_motion_adjoint_identity():
    W, H, F = 64, 48, 3
    xn, xm, bb = synth.make_motion(W, H, F, seed=9)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((F, H, W)) + 1j * rng.standard_normal((F, H, W))
    y = rng.standard_normal((F, H, W)) + 1j * rng.standard_normal((F, H, W))
    lhs = np.vdot(M.warp(x, xn, xm, bb), y)
    rhs = np.vdot(x, M.warp_adjoint(y, xn, xm, bb))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("W,H,F,amp", [(48, 40, 3, 1.2), (256, 256, 4, 1.2), (64, 56, 4, 3.0), (512, 128, 2, 1.2)])
def test_synthetic_motion_stays_inside_the_image(W, H, F, amp):
    """synth.make_motion: every rectangle entry's target and interpolation
    corners are inside the image (so the kernels never report status 5), and
    the meshes have the reference's layouts and 1-based values."""
    xn, xm, bb = synth.make_motion(W, H, F, seed=1, amplitude=amp)
    assert xn.shape == (2, F, H, W) and xn.dtype == np.float32
    assert xm.shape == (2, W, H) and xm.dtype == np.int32
    r1, r2 = M.rect(W, H, bb)
    assert r1.min() >= 0 and r1.max() < H and r2.min() >= 0 and r2.max() < W
    nh = xn[0][:, r1[:, None], r2[None, :]] - 1
    nv = xn[1][:, r1[:, None], r2[None, :]] - 1
    assert np.floor(nh).min() >= 0 and np.floor(nh).max() + 1 < W
    assert np.floor(nv).min() >= 0 and np.floor(nv).max() + 1 < H
    assert xm[0].min() == 1 and xm[0].max() == W and xm[1].min() == 1 and xm[1].max() == H
