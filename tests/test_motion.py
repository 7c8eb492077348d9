"""Motion-compensation oracle (oracle/motion.py) against the reference's own
interpolator / adjointInterpolator / initZeroRect / copyDataGPU kernels
compiled for the host, and the adjoint identity of the pair."""
from __future__ import annotations

import numpy as np
import pytest

from opencliper_gb300 import synth
from oracle import motion as M
from oracle import refkernels as K

pytestmark = pytest.mark.skipif(K.build() is None, reason="reference kernel sources not available")


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
