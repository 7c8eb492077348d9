"""CPU checks of the oracle itself: drand48 against libc, the power-method
reformulation used by the GPU against the literal restatement, operator
conventions and adjoint identities, the reference's stopping-rule quirks, and
the committed golden vectors."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

from oracle import drand48
from oracle import nesta_ref as R
from tests.conftest import ROOT, rel_l2


def test_drand48_restatement_matches_libc():
    a, sa = drand48.libc_sequence(20000)
    b, sb = drand48.lcg_sequence(20000)
    assert np.array_equal(a, b) and sa == sb
    a2, _ = drand48.libc_sequence(7, sa)
    b2, _ = drand48.lcg_sequence(7, sb)
    assert np.array_equal(a2, b2)


def test_drand48_jump_matches_iteration():
    x = drand48.DEFAULT_STATE
    for _ in range(1000):
        x = (drand48.A * x + drand48.C) & drand48.MASK
    ja, jc = drand48.jump(1000)
    assert (ja * drand48.DEFAULT_STATE + jc) & drand48.MASK == x


def _normest_per_pixel(F, H, W, state=drand48.DEFAULT_STATE):
    """Per-pixel form used by the GPU kernel: e_1 = ||r||, e_{m+1} = ||D b_m||/||b_m||."""
    N = H * W
    vals, _ = drand48.lcg_sequence(N * F, state)
    r = vals.astype(np.float32).astype(np.float64).reshape(F, N)
    A, B = [np.sum(r * r)], [0.0]
    b = r - np.roll(r, -1, axis=0)
    for _ in range(1, 100):
        d = b - np.roll(b, 1, axis=0)
        A.append(np.sum(b * b))
        B.append(np.sum(d * d))
        b = (d - np.roll(d, -1, axis=0)) * 0.25
    e, e0, cnt = np.float32(np.sqrt(np.float32(N * F))), np.float32(0), 0
    while abs(e - e0) > np.float32(1e-3) * e and cnt < 100:
        e0 = e
        e = np.float32(np.sqrt(A[0])) if cnt == 0 else np.float32(np.sqrt(B[cnt] / A[cnt]))
        cnt += 1
    return e, cnt


@pytest.mark.parametrize("F,H,W", [(2, 8, 8), (3, 8, 16), (5, 16, 16), (8, 16, 24), (20, 32, 32), (40, 16, 8)])
def test_normest_per_pixel_form_matches_literal(F, H, W):
    e_lit, c_lit, _ = R.normest(F, H, W, "f64")
    e_pix, c_pix = _normest_per_pixel(F, H, W)
    assert c_lit == c_pix
    assert abs(e_lit - e_pix) <= 2e-6 * e_lit


def test_normest_uses_libc_sequence():
    e1, c1, s1 = R.normest(4, 8, 8, "f32", use_libc=True)
    e2, c2, s2 = R.normest(4, 8, 8, "f32", use_libc=False)
    assert (e1, c1, s1) == (e2, c2, s2)


def test_ttv_adjoint_identity():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((5, 8, 8)) + 1j * rng.standard_normal((5, 8, 8))
    u = rng.standard_normal((5, 8, 8)) + 1j * rng.standard_normal((5, 8, 8))
    lhs = np.vdot(R.ttv(x, True), u)
    rhs = -np.vdot(x, R.ttv(u, False))  # the adjoint kernel computes -D^T
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)


def test_encode_adjoint_identity():
    rng = np.random.default_rng(1)
    F, C, H, W = 3, 2, 16, 24
    x = rng.standard_normal((F, H, W)) + 1j * rng.standard_normal((F, H, W))
    k = rng.standard_normal((F, C, H, W)) + 1j * rng.standard_normal((F, C, H, W))
    S = rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))
    mask = (rng.random((F, H, W)) > 0.4).astype(np.uint8) * 255
    lhs = np.vdot(R.encode(x, S, mask), k)
    rhs = np.vdot(x, R.encode_adjoint(R.apply_mask(k, mask), S))
    assert abs(lhs - rhs) < 1e-6 * abs(lhs)


def test_fft_conventions():
    rng = np.random.default_rng(2)
    a = rng.standard_normal((2, 8, 16)) + 1j * rng.standard_normal((2, 8, 16))
    assert rel_l2(R.fft2(R.fft2(a, True), False), a) < 1e-12
    assert abs(R.fft2(a, True)[0, 0, 0] - a[0].sum()) < 1e-9  # forward unscaled, DC at index 0


def test_rowmask_to_pixelmask():
    rm = np.array([[1, 0, 1, 1]], np.uint32)
    pm = R.rowmask_to_pixelmask(rm, 8)
    assert pm.shape == (1, 4, 8) and pm.dtype == np.uint8
    assert (pm[0, 0] == 255).all() and (pm[0, 1] == 0).all()
    with pytest.raises(ValueError):
        R.rowmask_to_pixelmask(np.array([[2]], np.uint32), 8)


def _tiny():
    from opencliper_gb300 import synth
    return synth.make_problem(16, 16, 4, 2, 2, seed=3)


def test_stoptest_quirk_second_hit_ends_loop():
    """NestaUp.cpp:799-824: the first qp <= tolVar skips the fmean update and
    sets qpDone; the second sets k = maxIter, so one more update runs with
    apk = (maxIter+1)/2 and the loop ends.  With tolVar so large that every
    test passes, each outer loop runs exactly miniter + 2 iterations."""
    p = _tiny()
    prm = R.NestaParams(maxIntIter=3, maxIter=100, stoptest=1, miniter=4, tolVar=1e30)
    r = R.nesta(p.y, p.S, p.mask, prm, "f32")
    assert r.stats["inner_iters"] == 3 * (4 + 2)


def test_stoptest_zero_runs_fixed_iterations():
    p = _tiny()
    prm = R.NestaParams(maxIntIter=2, maxIter=9, stoptest=0)
    r = R.nesta(p.y, p.S, p.mask, prm, "f32")
    assert r.stats["inner_iters"] == 18


def test_tolvar_written_back_like_reference():
    p = _tiny()
    prm = R.NestaParams(maxIntIter=4, maxIter=3, stoptest=0, tolVar=3e-4)
    r = R.nesta(p.y, p.S, p.mask, prm, "f32")
    # tolVar = 0.1 * gammat^maxIntIter == the requested tolVar (float rounding)
    assert abs(r.stats["tolVar_final"] - 3e-4) < 1e-9


def test_f32_close_to_f64_on_small_problem():
    p = _tiny()
    prm = R.NestaParams(maxIntIter=1, maxIter=20, stoptest=0, mu_f=1e-3)
    r32 = R.nesta(p.y, p.S, p.mask, prm, "f32")
    r64 = R.nesta(p.y, p.S, p.mask, prm, "f64")
    assert R.nrmse(r32.x, r64.x) < 1e-4


GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.mark.parametrize("name", sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz")) if os.path.isdir(GOLDEN) else [])
def test_oracle_reproduces_golden(name):
    d = np.load(os.path.join(GOLDEN, name))
    kind = str(d["kind"])
    if kind == "drand48":
        v, st = drand48.lcg_sequence(int(d["n"]), int(d["state"]))
        assert np.array_equal(v, d["values"]) and st == int(d["new_state"])
    elif kind == "nesta":
        prm = R.NestaParams(**{k: d["prm_" + k].item() for k in R.NestaParams.__dataclass_fields__})
        r = R.nesta(d["y"], d["S"], d["mask"], prm, str(d["precision"]), rand_state=int(d["rand_state"]))
        tol = 1e-12 if str(d["precision"]) == "f64" else 1e-6
        assert rel_l2(r.x, d["x"]) < tol
        assert r.stats["inner_iters"] == int(d["inner_iters"])
    elif kind == "simple":
        assert rel_l2(R.simple_recon(d["y"], d["S"]), d["x"]) < 1e-6
    elif kind == "refkernels":
        x, k, S = d["x"].astype(np.complex128), d["k"].astype(np.complex128), d["S"].astype(np.complex128)
        assert rel_l2(R.ttv(x, True), d["ttv_fwd"]) < 1e-6 and rel_l2(R.ttv(x, False), d["ttv_adj"]) < 1e-6
        assert rel_l2(R.normalize(x, float(d["mu"])), d["normalize"]) < 1e-6
        assert rel_l2(R.sensmul(x, S, False), d["sensmul_x"]) < 1e-6
        assert rel_l2(R.sensmul(k, S, True), d["sensmul_k_conj"]) < 1e-6
        assert rel_l2(R.coilsum(k), d["coilsum"]) < 1e-6
        assert np.array_equal(R.apply_mask(d["k"], d["mask"]), d["mask_k"])
        assert rel_l2(R.complex_abs2(k), d["abs2"]) < 1e-6 and rel_l2(R.complex_abs(x), d["abs"]) < 1e-6
    elif kind == "registration":
        from oracle import registration as RG
        prm = {k[4:]: (tuple(d[k]) if d[k].ndim else d[k].item()) for k in d.files if k.startswith("prm_")}
        r = RG.Registration(int(d["N"]), int(d["F"]), **prm).run(d["images"])
        assert r["iterations"] == int(d["iterations"])
        sys.path.insert(0, GOLDEN)
        import make_golden
        tol = make_golden.REG_T_TOL.get(name, 5e-6)
        assert np.abs(r["T"] - d["T"]).max() <= tol * np.abs(d["T"]).max() + 1e-6
    else:
        raise AssertionError(kind)


@pytest.mark.parametrize("prm", [
    dict(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=30, stoptest=0, miniter=7, tolVar=3e-4),
    dict(lambda_i=1e-2, mu_f=3e-4, La=1.0, maxIntIter=4, maxIter=100, stoptest=1, miniter=7, tolVar=3e-4),
])
def test_torch_fp64_restatement_matches_numpy_fp64(prm):
    """oracle/nesta_torch.py (the FP64 oracle for large workloads, run on the
    GPU by the accuracy tests) against nesta_ref's FP64 mode on the CPU."""
    pytest.importorskip("torch")
    from opencliper_gb300 import synth
    from oracle import nesta_ref as R
    from oracle import nesta_torch as RT
    p = synth.make_problem(40, 32, 5, 3, 4, seed=17)
    ref = R.nesta(p.y, p.S, p.mask, R.NestaParams(**prm), "f64")
    x, st = RT.nesta_f64(p.y, p.S, p.mask, R.NestaParams(**prm))
    assert R.nrmse(x, ref.x) < 1e-11
    assert st["inner_iters"] == ref.stats["inner_iters"]
    assert st["normest_iters"] == ref.stats["normest_iters"]
    assert st["rand_state"] == ref.stats["rand_state"]
    for k in ("normU", "lambda_", "mu0", "mu_final", "fx_final"):
        assert abs(st[k] - ref.stats[k]) <= 1e-10 * abs(ref.stats[k]), k
