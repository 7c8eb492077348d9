"""GroupwiseRegistration on the GPU (gbn_registration_run) against the
fixtures of the reference's own kernels (tests/golden/registration_*.npz,
made by oracle/refkernels/registration_host.hpp), the restatement in
oracle/registration.py for the starting-displacement path, and the hand-off
to the motion-compensated solve."""
import os
import sys

import numpy as np
import pytest

from opencliper_gb300 import api, synth
from opencliper_gb300._abi import GbnError

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu

CASES = [c[0] for c in make_golden.REG_CASES]


def _load(name):
    return dict(np.load(os.path.join(HERE, "golden", name)))


def _params(d, **over):
    kw = {k[4:]: (tuple(d[k]) if d[k].ndim else d[k].item()) for k in d if k.startswith("prm_")}
    kw.update(over)
    return api.registration_params(**kw)


def _run(ctx, images, prm, T_init=None):
    x = ctx.to_device(np.ascontiguousarray(images, np.complex64))
    tin = None if T_init is None else ctx.to_device(np.ascontiguousarray(T_init, np.float32))
    r = api.registration(ctx, x, prm, tin)
    return {k: (v.get() if isinstance(v, api.DeviceArray) else v) for k, v in r.items()}


@pytest.mark.parametrize("name", CASES)
def test_matches_reference_kernels(ctx, name):
    """Same iterations, weight and bounding box; T and the deformed mesh to
    float rounding of the reference kernels' results (the GPU sums the metric
    and |Dif| in a different order, and leaves out the reference's
    regularisation gradient, which the frame-mean projection cancels)."""
    d = _load(name)
    r = _run(ctx, d["images"], _params(d))
    assert r["status"] == 0
    assert r["iterations"] == int(d["iterations"])
    assert list(r["bound_box"]) == list(d["bb"])
    assert r["cp"] == int(d["C0"]) and r["area"] == int(d["areaX"])
    assert r["Wn"] == pytest.approx(float(d["Wn"]), rel=1e-6)
    scale = np.abs(d["T"]).max()
    tol = make_golden.REG_T_TOL.get(name, 1e-5)
    assert np.abs(r["T"] - d["T"]).max() <= tol * scale + 1e-6, np.abs(r["T"] - d["T"]).max()
    assert np.abs(r["xn"] - d["xn"]).max() <= make_golden.REG_XN_TOL.get(name, 5e-5)
    np.testing.assert_allclose(r["H"], d["H"], rtol=make_golden.REG_H_TOL.get(name, 1e-5))
    N = int(d["N"])
    xm = r["xmesh"]
    np.testing.assert_array_equal(xm[0], np.arange(N)[:, None] + 1 + 0 * np.arange(N)[None, :])
    np.testing.assert_array_equal(xm[1], np.arange(N)[None, :] + 1 + 0 * np.arange(N)[:, None])


def test_starting_displacements(ctx):
    """A later motion iteration (TData given) against the restatement."""
    from oracle import registration as RG
    d = _load(CASES[0])
    kw = {k[4:]: (tuple(d[k]) if d[k].ndim else d[k].item()) for k in d if k.startswith("prm_")}
    kw["nmax"] = 3
    ref = RG.Registration(int(d["N"]), int(d["F"]), **kw).run(d["images"], T_init=d["T"])
    r = _run(ctx, d["images"], api.registration_params(**kw), T_init=d["T"])
    assert r["iterations"] == ref["iterations"]
    assert np.abs(r["T"] - ref["T"]).max() <= 1e-5 * np.abs(ref["T"]).max() + 1e-6
    np.testing.assert_allclose(r["H"], ref["H"], rtol=1e-5)


def test_deterministic(ctx):
    d = _load(CASES[1])
    a = _run(ctx, d["images"], _params(d))
    b = _run(ctx, d["images"], _params(d))
    np.testing.assert_array_equal(a["T"], b["T"])
    np.testing.assert_array_equal(a["xn"], b["xn"])


@pytest.mark.parametrize("over,code", [(dict(radius=0), -2), (dict(E=4), -2), (dict(Dp=(4, 3)), -2),
                                       (dict(nmax=0), -1), (dict(radius=60), -2)])
def test_refused(ctx, over, code):
    d = _load(CASES[0])
    with pytest.raises(GbnError) as e:
        _run(ctx, d["images"], _params(d, **over))
    assert e.value.code == code


def test_refuses_zero_frames(ctx):
    with pytest.raises(GbnError) as e:
        _run(ctx, np.zeros((4, 64, 64), np.complex64), api.registration_params(radius=12, nmax=2))
    assert e.value.code == -1


def test_refuses_two_frames(ctx):
    img = synth.phantom_series(64, 64, 2, np.random.default_rng(1))
    with pytest.raises(GbnError):
        _run(ctx, img, api.registration_params(radius=12, nmax=2))


def test_feeds_motion_compensated_solve(ctx):
    """MRIRecon's motion loop (MRIRecon.cpp:246-282): register a plain
    reconstruction, then solve again with its mesh (ArgumentsMotionCompensation)."""
    W = H = 64
    F, Cc, R = 6, 4, 4
    p = synth.make_problem(W, H, F, Cc, R, seed=31)
    y, S, m = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
    prob = api.Problem(ctx, y, S, m)
    x = ctx.zeros((F, H, W), np.complex64)
    prm = api.nesta_params(maxIntIter=1, maxIter=20, stoptest=0)
    st0 = prob.run(prm, x)
    assert st0["status"] == 0
    reg = api.registration(ctx, x, api.registration_params(radius=12, nmax=4, W=0.05))
    assert reg["status"] == 0 and reg["iterations"] >= 1
    prob.set_motion(reg["xn"], reg["xmesh"], reg["bound_box"])
    st1 = prob.run(prm, x)
    assert st1["status"] == 0
    assert np.isfinite(x.get()).all()


def test_full_size_against_restatement(ctx):
    """The reference's default configuration at the MRIRecon size (256 x 256,
    20 frames, radius 40, 23 x 23 control points): two iterations against the
    restatement (seconds of numpy), then the full 100-iteration run's
    properties: status 0, the metric falls overall, T and xn finite."""
    from oracle import registration as RG
    img = synth.phantom_series(256, 256, 20, np.random.default_rng(41))
    kw = dict(nmax=2)
    ref = RG.Registration(256, 20, **kw).run(img)
    r = _run(ctx, img, api.registration_params(**kw))
    assert r["iterations"] == ref["iterations"] == 2
    assert np.abs(r["T"] - ref["T"]).max() <= 1e-5 * np.abs(ref["T"]).max() + 1e-6
    np.testing.assert_allclose(r["H"], ref["H"], rtol=1e-5)
    full = _run(ctx, img, api.registration_params())
    assert full["status"] == 0 and full["cp"] == 23
    assert full["H"][-1] < full["H"][0]
    assert np.isfinite(full["T"]).all() and np.isfinite(full["xn"]).all()


def test_continuation_in_place(ctx):
    """T_init may be the output array itself (the C ABI's d_T_init == d_T)."""
    import ctypes as C
    from opencliper_gb300._abi import RegistrationStats, call
    d = _load(CASES[0])
    prm = _params(d, nmax=3)
    x = ctx.to_device(d["images"])
    ref = api.registration(ctx, x, prm, ctx.to_device(d["T"]))
    N, F = int(d["N"]), int(d["F"])
    T = ctx.to_device(np.ascontiguousarray(d["T"], np.float32))
    xn = ctx.empty((2, F, N, N), np.float32)
    xm = ctx.empty((2, N, N), np.int32)
    st = RegistrationStats()
    call("gbn_registration_run", ctx.handle, x.ptr, N, F, C.byref(prm), T.ptr, T.ptr, xn.ptr, xm.ptr, None,
         C.byref(st))
    np.testing.assert_array_equal(T.get(), ref["T"].get())
    np.testing.assert_array_equal(xn.get(), ref["xn"].get())
