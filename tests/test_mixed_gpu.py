"""Mixed-precision form (GBN_PRECISION_MIXED): the forward column transform
runs on the tensor cores with split fp16 operands (hi + lo) and FP32
accumulation.  Its error per product is a few 1e-7, the same class as FP32
arithmetic, so the result must stay as close to the FP64 oracle as the FP32
restatement does, with a small allowance for the different rounding:
NRMSE(mixed, f64) <= 3 * NRMSE(f32 oracle, f64) + 1e-5.  Ragged shapes cover
H not a multiple of 16 (padded K chunks), W not a multiple of 32 (masked
columns), C not a multiple of 4 (masked coils) and uneven kept rows."""
from __future__ import annotations

import numpy as np
import pytest

import opencliper_gb300 as g
from opencliper_gb300 import synth
from oracle import drand48
from oracle import nesta_ref as R

pytestmark = pytest.mark.gpu

FIXED = dict(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=30, stoptest=0, miniter=7, tolVar=3e-4)
DRIVER = dict(lambda_i=1e-2, mu_f=3e-4, La=1.0, maxIntIter=3, maxIter=40, stoptest=1, miniter=5, tolVar=3e-4)

@pytest.fixture(autouse=True)
def _tensor_core_forward(ctx):
    """These shapes are small enough that the automatic choice would run their
    groups on the FP32 kernels: force the tensor-core forward pass."""
    ctx.set_tuning("mixed_fwd_tc", 1)
    yield
    ctx.set_tuning("mixed_fwd_tc", -1)


CASES = [(32, 32, 6, 4, 4, FIXED), (48, 40, 5, 3, 4, FIXED), (64, 64, 8, 5, 2, FIXED), (40, 24, 3, 7, 2, FIXED),
         (96, 64, 6, 6, 4, DRIVER)]


@pytest.mark.parametrize("adjoint_tc", [0, 1])
@pytest.mark.parametrize("W,H,F,C,Rr,prm", CASES + [(32, 24, 4, 19, 2, FIXED)])
def test_mixed_against_oracle(ctx, W, H, F, C, Rr, prm, adjoint_tc):
    """Forward column pass on the tensor cores, and optionally the adjoint one
    (C = 19 takes two coil groups through tensor memory)."""
    ctx.set_tuning("mixed_adjoint_tc", adjoint_tc)
    p = synth.make_problem(W, H, F, C, Rr, seed=40 + W + C)
    dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
    prob = g.Problem(ctx, dy, dS, dm)
    x = ctx.empty((F, H, W), np.complex64)
    s0 = drand48.seed16v_to_state(ctx.rand48())
    b = g.Batch(ctx, [prob], g.nesta_params(**prm), [x], precision=g.PRECISION_MIXED)
    ctx.set_tuning("mixed_adjoint_tc", 0)
    b.launch()
    got = x.get()
    st = b.stats(0)
    b.close()
    prob.close()
    r64 = R.nesta(p.y, p.S, p.mask, R.NestaParams(**prm), "f64", rand_state=s0)
    r32 = R.nesta(p.y, p.S, p.mask, R.NestaParams(**prm), "f32", rand_state=s0)
    e_mx, e_32 = R.nrmse(got, r64.x), R.nrmse(r32.x, r64.x)
    print(f"NRMSE mixed/f64 {e_mx:.3e}  f32-oracle/f64 {e_32:.3e}")
    assert st["status"] == 0
    assert np.isfinite(got).all()
    assert e_mx <= 3.0 * e_32 + 1e-5
    assert st["inner_iters"] == r32.stats["inner_iters"]


def test_mixed_batch_uneven_matches_members(ctx):
    """Members of a mixed batch give the same images as mixed batches of one."""
    cases = [(32, 32, 6, 4, 4), (32, 32, 3, 7, 2), (48, 40, 5, 3, 4), (32, 32, 9, 2, 4)]
    items = []
    for k, (W, H, F, C, Rr) in enumerate(cases):
        p = synth.make_problem(W, H, F, C, Rr, seed=600 + k)
        dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
        items.append((g.Problem(ctx, dy, dS, dm), ctx.empty((F, H, W), np.complex64), (dy, dS, dm)))
    prm = g.nesta_params(**FIXED)
    s0 = 0x00AB00CD00EF
    singles = []
    state = s0
    for prob, x, _ in items:
        ctx.seed48(drand48.state_to_seed16v(state))
        b = g.Batch(ctx, [prob], prm, [x], precision=g.PRECISION_MIXED)
        b.launch()
        singles.append(x.get())
        b.close()
        state = drand48.seed16v_to_state(ctx.rand48())
    ctx.seed48(drand48.state_to_seed16v(s0))
    b = g.Batch(ctx, [it[0] for it in items], prm, [it[1] for it in items], precision=g.PRECISION_MIXED)
    b.capture()
    b.launch()
    for (prob, x, _), ref in zip(items, singles):
        assert np.array_equal(x.get(), ref)
    b.close()
    for prob, _, _ in items:
        prob.close()


def test_mixed_rejects_too_many_kept_rows(ctx):
    p = synth.make_problem(32, 320, 2, 2, 2, seed=5)  # 160 kept rows per frame > 128
    dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
    prob = g.Problem(ctx, dy, dS, dm)
    x = ctx.empty((2, 320, 32), np.complex64)
    with pytest.raises(g.GbnError):
        g.Batch(ctx, [prob], g.nesta_params(**FIXED), [x], precision=g.PRECISION_MIXED)
    prob.close()


@pytest.mark.parametrize("W,H,F,C,Rr", [(48, 40, 5, 3, 4), (32, 384, 3, 3, 8)])
def test_mixed_forward_choice_per_group(ctx, W, H, F, C, Rr):
    """mixed_fwd_tc = 0 runs a mixed batch's groups on the plain FP32 kernels
    (the same image as an FP32 batch, bit for bit), and so does the automatic
    choice for row masks at any H (the FP32 row-local iteration beats the
    tensor-core forms); mixed_fwd_tc = 1 runs the row-local iteration on the
    tensor cores."""
    p = synth.make_problem(W, H, F, C, Rr, seed=91)
    dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
    prob = g.Problem(ctx, dy, dS, dm)
    x = ctx.empty((F, H, W), np.complex64)
    prm = g.nesta_params(**FIXED)
    imgs, paths = [], []
    for prec, tc in ((g.PRECISION_FP32, 1), (g.PRECISION_MIXED, 0), (g.PRECISION_MIXED, -1), (g.PRECISION_MIXED, 1)):
        ctx.set_tuning("mixed_fwd_tc", tc)
        ctx.seed48(drand48.state_to_seed16v(drand48.DEFAULT_STATE))
        b = g.Batch(ctx, [prob], prm, [x], precision=prec)
        b.launch()
        imgs.append(x.get())
        info = b.group_info(0)
        assert (info["W"], info["H"], info["members"]) == (W, H, [0])
        paths.append(info["path"])
        b.close()
    assert paths == ["row_local", "row_local", "row_local", "row_local_tc"]
    prob.close()
    assert np.array_equal(imgs[0], imgs[1]) and np.array_equal(imgs[0], imgs[2])
    assert not np.array_equal(imgs[0], imgs[3])  # the tensor-core transforms round differently
    assert R.nrmse(imgs[3], imgs[0]) < 1e-3


def test_mixed_partly_sampled_rows_three_pass(ctx):
    """A pixel mask with partly sampled rows needs the row pass, so a mixed
    batch keeps the three-pass form (tensor-core forward transform)."""
    rng = np.random.default_rng(3)
    p = synth.make_problem(48, 40, 5, 3, 4, seed=17)
    p.mask = ((rng.random(p.mask.shape) > 0.6) * 255).astype(np.uint8)
    p.y = np.where(p.mask[:, None] == 0, 0, p.y).astype(np.complex64)
    dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
    prob = g.Problem(ctx, dy, dS, dm)
    x = ctx.empty((5, 40, 48), np.complex64)
    s0 = drand48.seed16v_to_state(ctx.rand48())
    b = g.Batch(ctx, [prob], g.nesta_params(**FIXED), [x], precision=g.PRECISION_MIXED)
    b.launch()
    got, st = x.get(), b.stats(0)
    assert b.group_info(0)["path"] == "three_pass_tc"
    with pytest.raises(g.GbnError):
        b.group_info(1)
    b.close()
    prob.close()
    r64 = R.nesta(p.y, p.S, p.mask, R.NestaParams(**FIXED), "f64", rand_state=s0)
    r32 = R.nesta(p.y, p.S, p.mask, R.NestaParams(**FIXED), "f32", rand_state=s0)
    e_mx, e_32 = R.nrmse(got, r64.x), R.nrmse(r32.x, r64.x)
    print(f"partly sampled rows: NRMSE mixed/f64 {e_mx:.3e}  f32-oracle/f64 {e_32:.3e}")
    assert st["status"] == 0 and np.isfinite(got).all()
    assert e_mx <= 3.0 * e_32 + 1e-5
