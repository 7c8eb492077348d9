"""Motion-compensated NESTA on the GPU: the warp and its adjoint against the
oracle, and the full solve (NestaUp with argsMC) against the FP64 / FP32
restatement started from the same image.  Both operators are gathers with
the reference kernels' rounding and match the oracle (an in-order scatter for
the adjoint) bit for bit.  With motion compensation the power method starts
from the interpolation's rounding residue on a constant image and converges
slowly; its norms are reduced in FP64 here and in float-then-FP64 by the
oracle, so ||U|| is compared to 2e-3 (one power-method step) and the stopping
step to one."""
from __future__ import annotations

import numpy as np
import pytest

import opencliper_gb300 as g
from opencliper_gb300 import api, synth
from oracle import drand48
from oracle import motion as M
from oracle import nesta_ref as R
from tests.conftest import rel_l2
from tests.test_nesta_gpu import LENGTHS, THREE_PASS_ONLY

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H,F,amp", [(48, 40, 3, 1.2), (128, 96, 5, 1.2), (64, 56, 4, 3.0)])
def test_motion_operators(ctx, W, H, F, amp):
    xn, xm, bb = synth.make_motion(W, H, F, seed=W, amplitude=amp)
    rng = np.random.default_rng(H)
    x = (rng.standard_normal((F, H, W)) + 1j * rng.standard_normal((F, H, W))).astype(np.complex64)
    dx, out = ctx.to_device(x), ctx.empty((F, H, W), np.complex64)
    dxn, dxm = ctx.to_device(xn), ctx.to_device(xm)
    api.op_motion(ctx, 1, dx, out, dxn, dxm, bb)  # forward (GBN_TTV_FORWARD): a gather, bit-exact
    assert np.array_equal(out.get(), M.warp(x, xn, xm, bb))
    api.op_motion(ctx, 0, dx, out, dxn, dxm, bb)  # adjoint: ordered gather, bit-exact with an in-order scatter
    assert np.array_equal(out.get(), M.warp_adjoint(x, xn, xm, bb))


def test_motion_rejects_bad_box(ctx):
    W, H, F = 32, 32, 2
    xn, xm, bb = synth.make_motion(W, H, F, seed=1)
    x = ctx.zeros((F, H, W), np.complex64)
    with pytest.raises(g.GbnError):
        api.op_motion(ctx, 1, x, x, ctx.to_device(xn), ctx.to_device(xm), [1, 1, W + 5, H])


FIXED_MC = dict(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=25, stoptest=0, miniter=7, tolVar=3e-4)
# continuation over three outer loops with the rolling-mean stopping test
DRIVER_MC = dict(lambda_i=1e-2, mu_f=3e-4, La=1.0, maxIntIter=3, maxIter=30, stoptest=1, miniter=5, tolVar=3e-4)


@pytest.mark.parametrize("W,H,F,C,Rr,prm", [(48, 40, 6, 3, 4, FIXED_MC), (64, 64, 8, 4, 4, FIXED_MC),
                                            (48, 40, 6, 3, 4, DRIVER_MC)])
def test_nesta_motion_compensated(ctx, W, H, F, C, Rr, prm):
    p = synth.make_problem(W, H, F, C, Rr, seed=W + F)
    xn, xm, bb = synth.make_motion(W, H, F, seed=F)
    dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
    prob = g.Problem(ctx, dy, dS, dm)
    x = ctx.empty((F, H, W), np.complex64)
    prob.run(g.nesta_params(**FIXED_MC), x)       # first reconstruction, without motion
    x0 = x.get()
    dxn, dxm = ctx.to_device(xn), ctx.to_device(xm)
    prob.set_motion(dxn, dxm, bb)
    s0 = drand48.seed16v_to_state(ctx.rand48())
    st = prob.run(g.nesta_params(**prm), x)       # starts from x0, the output's content
    got = x.get()
    ctx.seed48(drand48.state_to_seed16v(s0))      # the same solve again: deterministic
    x.set(x0)
    st2 = prob.run(g.nesta_params(**prm), x)
    assert np.array_equal(x.get(), got) and st2["normU"] == st["normU"]
    prob.close()
    assert st["status"] == 0
    r64 = R.nesta(p.y, p.S, p.mask, R.NestaParams(**prm), "f64", rand_state=s0, mc=(xn, xm, bb), x_init=x0)
    r32 = R.nesta(p.y, p.S, p.mask, R.NestaParams(**prm), "f32", rand_state=s0, mc=(xn, xm, bb), x_init=x0)
    e_gpu, e_32 = R.nrmse(got, r64.x), R.nrmse(r32.x, r64.x)
    print(f"MC NRMSE gpu/f64 {e_gpu:.3e}  f32-oracle/f64 {e_32:.3e}  normU {st['normU']:.5f} vs {r32.stats['normU']:.5f}")
    assert np.isfinite(got).all()
    assert abs(st["normU"] - r32.stats["normU"]) <= 2e-3 * r32.stats["normU"]
    assert abs(st["normest_iters"] - r32.stats["normest_iters"]) <= 1
    assert e_gpu <= 2.0 * e_32 + 2e-5
    assert st["inner_iters"] == r32.stats["inner_iters"]


def test_motion_row_local_matches_three_pass(ctx):
    """Row masks send the motion-compensated solve through the row-local
    iteration (k_mc_tv and M^T g, then the one-kernel data term and update);
    with the tuning knob off it runs the three-pass iteration.  The two agree
    to FP32 rounding over 20 iterations."""
    W, H, F, C, Rr = 64, 64, 8, 4, 6
    p = synth.make_problem(W, H, F, C, Rr, seed=31)
    xn, xm, bb = synth.make_motion(W, H, F, seed=5)
    dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
    prob = g.Problem(ctx, dy, dS, dm)
    x = ctx.empty((F, H, W), np.complex64)
    prob.run(g.nesta_params(**FIXED_MC), x)
    x0 = x.get()
    prob.set_motion(ctx.to_device(xn), ctx.to_device(xm), bb)
    prm = g.nesta_params(**{**FIXED_MC, "maxIter": 20})
    s0 = ctx.rand48()
    outs, sts, iters = [], [], []
    for rl in (1, 0):
        ctx.set_tuning("row_local", rl)
        ctx.seed48(s0)
        x.set(x0)
        ctx.profile(True)
        ctx.profile_reset()
        sts.append(prob.run(prm, x))
        iters.append(ctx.profile_read().get("iter", (0, 0.0))[0])
        ctx.profile(False)
        outs.append(x.get())
    ctx.set_tuning("row_local", 1)
    prob.close()
    assert iters[0] == 20 and iters[1] == 0
    assert sts[0]["status"] == 0 and sts[1]["status"] == 0
    assert sts[0]["inner_iters"] == sts[1]["inner_iters"] == 20
    err = R.nrmse(outs[0], outs[1])
    print(f"motion row-local vs three-pass: NRMSE {err:.3e}")
    assert 0 < err <= 1e-4


@pytest.mark.parametrize("H", [h for h in LENGTHS if h >= 16 and h not in THREE_PASS_ONLY])
def test_motion_row_local_every_column_length(ctx, H):
    """The motion-compensated row-local kernel (k_iter_cols<H, true>: the
    update reads M^T g instead of the neighbouring frames, in the operand
    prefetch or the batched loads as the length's budget chooses) at every
    column length that has a row-local form (from 16: the motion rectangle
    needs room inside the margins), against the three-pass iteration, 10
    iterations from the same starting image."""
    W, F, C = 64, 3, 3
    p = synth.make_problem(W, H, F, C, 8, seed=H + 1)
    xn, xm, bb = synth.make_motion(W, H, F, seed=H)
    dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
    prob = g.Problem(ctx, dy, dS, dm)
    x = ctx.empty((F, H, W), np.complex64)
    try:
        prob.run(g.nesta_params(**{**FIXED_MC, "maxIter": 10}), x)
        x0 = x.get()
        prob.set_motion(ctx.to_device(xn), ctx.to_device(xm), bb)
        prm = g.nesta_params(**{**FIXED_MC, "maxIter": 10})
        s0 = ctx.rand48()
        outs, sts, iters = [], [], []
        for rl in (1, 0):
            ctx.set_tuning("row_local", rl)
            ctx.seed48(s0)
            x.set(x0)
            ctx.profile(True)
            ctx.profile_reset()
            sts.append(prob.run(prm, x))
            iters.append(ctx.profile_read().get("iter", (0, 0.0))[0])
            ctx.profile(False)
            outs.append(x.get())
    finally:
        ctx.profile(False)
        ctx.set_tuning("row_local", 1)
        prob.close()
    assert iters[0] == 10 and iters[1] == 0
    assert sts[0]["status"] == 0 and sts[1]["status"] == 0
    assert sts[0]["inner_iters"] == sts[1]["inner_iters"] == 10
    assert np.isfinite(outs[0]).all()
    err = R.nrmse(outs[0], outs[1])
    print(f"H={H}: motion row-local vs three-pass NRMSE {err:.3e}")
    assert err <= 1e-5  # measured 4.6e-8 ... 6.4e-8
