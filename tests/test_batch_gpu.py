"""Batched tTV-NESTA (gbn_batch_*): uneven problems solved together, with and
without CUDA-graph capture.

Every reduction of the solver runs in a fixed order that does not depend on
which CTA did which piece of work or on the other problems of a launch, so a
batch must reproduce, bit for bit, the images of the same problems run one
after another through gbn_nesta_run from the same drand48 state.  Those
single runs are themselves checked against the oracle (test_nesta_gpu.py);
one batch member is also checked against the oracle here."""
from __future__ import annotations

import numpy as np
import pytest

import opencliper_gb300 as g
from opencliper_gb300 import synth
from oracle import drand48
from oracle import nesta_ref as R
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

FIXED = dict(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=30, stoptest=0, miniter=7, tolVar=3e-4)
DRIVER = dict(lambda_i=1e-2, mu_f=3e-4, La=1.0, maxIntIter=3, maxIter=40, stoptest=1, miniter=5, tolVar=3e-4)

# (W, H, F, C, R, params): two sizes shared by several members, uneven F and C,
# different iteration counts and continuation settings inside one group
CASES = [
    (32, 32, 6, 4, 4, FIXED),
    (48, 40, 5, 3, 4, DRIVER),
    (32, 32, 3, 7, 2, dict(FIXED, maxIter=17)),
    (32, 32, 9, 2, 4, DRIVER),
    (48, 40, 4, 5, 2, dict(FIXED, maxIter=45)),
    (64, 64, 8, 4, 6, FIXED),
]


def _state(ctx) -> int:
    return drand48.seed16v_to_state(ctx.rand48())


def _setup(ctx, cases, seed0=100):
    items = []
    for k, (W, H, F, C, Rr, prm) in enumerate(cases):
        p = synth.make_problem(W, H, F, C, Rr, seed=seed0 + k)
        dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
        prob = g.Problem(ctx, dy, dS, dm)
        items.append((p, prob, g.nesta_params(**prm), prm))
    return items


def _singles(ctx, items, state):
    ctx.seed48(drand48.state_to_seed16v(state))
    outs, stats = [], []
    for p, prob, prm, _ in items:
        F, C, H, W = p.y.shape
        x = ctx.empty((F, H, W), np.complex64)
        stats.append(prob.run(prm, x))
        outs.append(x.get())
    return outs, stats, _state(ctx)


def _batch_outputs(ctx, items):
    return [ctx.empty((p.y.shape[0], p.y.shape[2], p.y.shape[3]), np.complex64) for p, *_ in items]


def test_batch_matches_single_runs(ctx):
    items = _setup(ctx, CASES)
    s0 = drand48.DEFAULT_STATE
    ref, ref_stats, s1 = _singles(ctx, items, s0)
    outs = _batch_outputs(ctx, items)
    ctx.seed48(drand48.state_to_seed16v(s0))
    b = g.Batch(ctx, [it[1] for it in items], [it[2] for it in items], outs)
    b.launch()
    for i, (o, r) in enumerate(zip(outs, ref)):
        got = o.get()
        assert np.array_equal(got, r), f"member {i}: max |diff| {np.abs(got - r).max():.3e}"
        st = b.stats(i)
        for key in ("normU", "lambda_", "mu0", "inner_iters", "normest_iters", "kept_rows", "fx_final"):
            assert st[key] == ref_stats[i][key], (i, key)
    assert _state(ctx) == s1
    b.close()
    for _, prob, _, _ in items:
        prob.close()


def test_batch_member_against_oracle(ctx):
    items = _setup(ctx, CASES[:3], seed0=300)
    outs = _batch_outputs(ctx, items)
    s0 = _state(ctx)
    b = g.Batch(ctx, [it[1] for it in items], [it[2] for it in items], outs)
    b.launch()
    # member 1 starts W0*H0*F0 draws after the batch's start state
    p0 = items[0][0]
    p, _, _, prm = items[1]
    ja, jc = drand48.jump(p0.y.shape[0] * p0.y.shape[2] * p0.y.shape[3])
    rs = (ja * s0 + jc) & drand48.MASK
    r64 = R.nesta(p.y, p.S, p.mask, R.NestaParams(**prm), "f64", rand_state=rs)
    r32 = R.nesta(p.y, p.S, p.mask, R.NestaParams(**prm), "f32", rand_state=rs)
    got = outs[1].get()
    assert R.nrmse(got, r64.x) <= 2.0 * R.nrmse(r32.x, r64.x) + 5e-6
    assert b.stats(1)["inner_iters"] == r32.stats["inner_iters"]
    b.close()
    for _, prob, _, _ in items:
        prob.close()


def test_batch_graph_replays(ctx):
    items = _setup(ctx, CASES[:4], seed0=500)
    s0 = 0x0123456789AB
    ref0, _, s1 = _singles(ctx, items, s0)
    ref1, _, s2 = _singles(ctx, items, s1)
    outs = _batch_outputs(ctx, items)
    ctx.seed48(drand48.state_to_seed16v(s0))
    b = g.Batch(ctx, [it[1] for it in items], [it[2] for it in items], outs)
    b.capture()
    assert _state(ctx) == s0  # capturing runs nothing
    for ref, s_after in ((ref0, s1), (ref1, s2)):
        b.launch()
        for o, r in zip(outs, ref):
            assert np.array_equal(o.get(), r)
        assert _state(ctx) == s_after
    b.close()
    for _, prob, _, _ in items:
        prob.close()


def test_batch_splits_groups_beyond_64(ctx):
    cases = [(16, 16, 2, 1 + k % 3, 2, dict(FIXED, maxIter=4 + k % 5)) for k in range(67)]
    items = _setup(ctx, cases, seed0=900)
    ref, _, s1 = _singles(ctx, items, drand48.DEFAULT_STATE)
    outs = _batch_outputs(ctx, items)
    ctx.seed48(drand48.state_to_seed16v(drand48.DEFAULT_STATE))
    b = g.Batch(ctx, [it[1] for it in items], [it[2] for it in items], outs)
    b.launch()
    for o, r in zip(outs, ref):
        assert np.array_equal(o.get(), r)
    assert _state(ctx) == s1
    b.close()
    for _, prob, _, _ in items:
        prob.close()


def test_batch_rejects_bad_input(ctx):
    items = _setup(ctx, CASES[:2], seed0=700)
    probs = [it[1] for it in items]
    prms = [it[2] for it in items]
    outs = _batch_outputs(ctx, items)
    with pytest.raises(g.GbnError):
        g.Batch(ctx, probs, prms, outs, precision=g.PRECISION_MIXED + 5)
    with pytest.raises(g.GbnError):
        g.Batch(ctx, [probs[0], probs[0]], prms, outs)
    with pytest.raises(ValueError):
        g.Batch(ctx, probs, prms, outs[:1])
    for prob in probs:
        prob.close()


def test_maximum_sizes(ctx):
    """The largest supported shape (W = H = 512, 64 frames, the power method's
    frame limit): finite, no status, batched graph replay equal to the single
    run bit for bit, the mixed form within FP32-class distance of it, and the
    kept rows those of the masks."""
    W = H = 512
    F, Cc, Rr = 64, 4, 8
    p = synth.make_problem_device(ctx, W, H, F, Cc, Rr, seed=77)
    prm = g.nesta_params(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=10, stoptest=0, miniter=7,
                         tolVar=3e-4)
    prob = g.Problem(ctx, p.y, p.S, p.mask)
    x1, x2 = ctx.empty((F, H, W), np.complex64), ctx.empty((F, H, W), np.complex64)
    ctx.seed48(drand48.state_to_seed16v(drand48.DEFAULT_STATE))
    st = prob.run(prm, x1)
    assert st["status"] == 0 and st["kept_rows"] == int(p.rowmask.astype(bool).sum())
    a = x1.get()
    assert np.isfinite(a).all() and np.abs(a).max() > 0
    for prec, exact in ((g.PRECISION_FP32, True), (g.PRECISION_MIXED, False)):
        ctx.seed48(drand48.state_to_seed16v(drand48.DEFAULT_STATE))
        b = g.Batch(ctx, [prob], prm, [x2], precision=prec)
        b.capture()
        b.launch()
        assert b.stats(0)["status"] == 0
        c = x2.get()
        if exact:
            assert np.array_equal(a, c)
        else:
            assert rel_l2(c, a) < 1e-3
        b.close()
    prob.close()
    for d in (p.y, p.S, p.mask, x1, x2):
        d.free()


def test_batch_membership_guards(ctx):
    """While a batch holds a problem, resizing its row buffer and destroying it
    are refused (the batch's tables point into its buffers)."""
    p = synth.make_problem(32, 32, 4, 2, 4, seed=5)
    dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
    prob = g.Problem(ctx, dy, dS, dm)
    x = ctx.empty((4, 32, 32), np.complex64)
    b = g.Batch(ctx, [prob], g.nesta_params(maxIter=5, maxIntIter=1, stoptest=0), [x])
    with pytest.raises(g.GbnError):
        prob.fit_rows(0)
    from opencliper_gb300._abi import call
    with pytest.raises(g.GbnError):
        call("gbn_problem_destroy", prob.handle)
    b.close()
    assert prob.fit_rows(0) == int(p.rowmask.astype(bool).sum())
    prob.close()
