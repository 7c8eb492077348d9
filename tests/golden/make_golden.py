"""Generates the golden fixtures of tests/golden/ (small, committed).

drand48_libc.npz : values drawn from the C library's drand48 after resetting
                   it to its default state (the sequence NestaUp's power-method
                   restart consumes, NestaUp.cpp:369-385)
nesta_*.npz      : inputs, parameters and outputs of the CPU restatement of
                   NestaUp::launch for small seeded problems
simple_*.npz     : SimpleMRIRecon on a small fully sampled problem
ops_refkernels.npz : outputs of the reference's own operator kernels
                   (src/kernels/*.cl compiled for the host by oracle/refkernels)
                   on seeded inputs; written only where the reference sources
                   are available
registration_*.npz : GroupwiseRegistration run on the host with the
                   reference's own kernels (oracle/refkernels/
                   registration_host.hpp) on seeded cine phantoms: inputs,
                   parameters, T, xn, the metric per iteration; written only
                   where the reference sources are available

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import drand48  # noqa: E402
from oracle import nesta_ref as R  # noqa: E402
from opencliper_gb300 import synth  # noqa: E402


def save(name, **kw):
    np.savez_compressed(os.path.join(HERE, name), **kw)
    print("wrote", name)


def nesta_case(name, p, prm: R.NestaParams, precision):
    r = R.nesta(p.y, p.S, p.mask, prm, precision)
    save(name, kind="nesta", precision=precision, y=p.y, S=p.S, mask=p.mask, x=r.x,
         rand_state=drand48.DEFAULT_STATE, inner_iters=r.stats["inner_iters"], normU=r.stats["normU"],
         **{"prm_" + k: getattr(prm, k) for k in R.NestaParams.__dataclass_fields__})


def main():
    vals, st = drand48.libc_sequence(4096)
    save("drand48_libc.npz", kind="drand48", n=4096, state=drand48.DEFAULT_STATE, values=vals, new_state=st)
    # continuation quirks: defaults of tests/MRIRecon.cpp:105-114 on a small cine problem
    p = synth.make_problem(24, 16, 4, 3, 2, seed=11)
    nesta_case("nesta_24x16x4c3_defaults_f64.npz", p, R.NestaParams(maxIter=40), "f64")
    nesta_case("nesta_24x16x4c3_defaults_f32.npz", p, R.NestaParams(maxIter=40), "f32")
    # fixed iterations, random pixel mask, data outside the mask kept by the solver
    rng = np.random.default_rng(5)
    q = synth.make_problem(32, 24, 3, 2, 3, seed=12)
    q.mask = ((rng.random(q.mask.shape) > 0.5) * 255).astype(np.uint8)
    q.y = q.y.copy()
    q.y[:, :, 5, :] += (0.01 * (rng.standard_normal((3, 2, 32)) + 1j * rng.standard_normal((3, 2, 32)))).astype(np.complex64)
    nesta_case("nesta_32x24x3c2_pixmask_f64.npz", q,
               R.NestaParams(lambda_i=0.01, mu_f=1e-3, maxIntIter=1, maxIter=25, stoptest=0), "f64")
    s = synth.make_fully_sampled(32, 32, 4, seed=13)
    save("simple_32x32c4.npz", kind="simple", y=s.y, S=s.S, x=R.simple_recon(s.y.astype(np.complex128),
                                                                          s.S.astype(np.complex128)))


def refkernel_ops():
    from oracle import refkernels as K
    if K.build() is None or not K.available():
        print("reference kernel sources unavailable: ops_refkernels.npz not regenerated")
        return
    rng = np.random.default_rng(77)
    W, H, F, C = 24, 16, 3, 2
    c = lambda shape: (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    x, k, S = c((F, H, W)), c((F, C, H, W)), c((C, H, W))
    mask = ((rng.random((F, H, W)) > 0.5) * 255).astype(np.uint8)
    save("ops_refkernels.npz", kind="refkernels", x=x, k=k, S=S, mask=mask, mu=np.float32(0.6),
         ttv_fwd=K.ttv(x, True), ttv_adj=K.ttv(x, False), normalize=K.normalize(x, 0.6),
         sensmul_x=K.sensmul(x, S, False), sensmul_k_conj=K.sensmul(k, S, True), coilsum=K.coilsum(k),
         mask_k=K.apply_mask(k, mask), abs2=K.abs2(k), abs=K.cabs(x), rss=K.rss(k))


REG_CASES = [
    # name, N, F, seed, parameters (the rest are tests/MRIRecon.cpp:121-129)
    ("registration_64x4_circle.npz", 64, 4, 21, dict(radius=12, nmax=6, W=0.05)),
    # a weight of at least 1 makes sumLambda() non-zero, so the smoothness terms enter the metric
    ("registration_64x5_lambda.npz", 64, 5, 22, dict(radius=14, nmax=5, W=0.05, lambda_=(0.01, 0.02, 0.1, 1.5))),
    ("registration_96x6_circle.npz", 96, 6, 23, dict(radius=20, nmax=4, W=0.2, flagW=False)),
    # stopCondition fires before nmax: |Dif| < et 2F and a metric change below eh H0 at iteration 4
    ("registration_64x4_stop.npz", 64, 4, 24, dict(radius=12, nmax=12, W=0.05, et=0.5, eh=0.05)),
    # linear and quadratic splines (creabspline.cpp's odd and even control ranges)
    ("registration_64x4_e1.npz", 64, 4, 25, dict(radius=12, nmax=5, W=0.05, E=1)),
    ("registration_64x4_e2.npz", 64, 4, 25, dict(radius=12, nmax=5, W=0.05, E=2, lambda_=(0.0, 0.0, 0.0, 0.5))),
    # quadratic splines with the default weights: the order-2 derivative table (b1spline2's
    # 42 x) makes the frame-broadcast regularisation term large, and its cancellation in the
    # projected update leaves a rounding residue of ~1e-4 in T (REG_T_TOL)
    ("registration_64x4_e2_lambda.npz", 64, 4, 25, dict(radius=12, nmax=5, W=0.05, E=2)),
]
# tolerances where they are not a few roundings: T relative to max |T_ref|, xn in
# pixels, H relative
REG_T_TOL = {"registration_64x4_e2_lambda.npz": 5e-4}
REG_XN_TOL = {"registration_64x4_e2_lambda.npz": 1e-3}
REG_H_TOL = {"registration_64x4_e2_lambda.npz": 2e-5}


def registration_inputs(N, F, seed):
    return synth.phantom_series(N, N, F, np.random.default_rng(seed))


def registration_cases():
    from oracle import refkernels as K
    if K.build() is None or not K.available():
        print("reference kernel sources unavailable: registration_*.npz not regenerated")
        return
    for name, N, F, seed, kw in REG_CASES:
        prm = dict(radius=40, E=3, Dp=(4, 4), nmax=100, et=0.01, eh=0.005, lambda_=(0.0, 0.005, 0.0, 0.5), W=1.0,
                   flagW=True)
        prm.update(kw)
        img = registration_inputs(N, F, seed)
        r = K.registration(img, **prm)
        save(name, kind="registration", images=img, N=N, F=F, seed=seed,
             **{"prm_" + k: np.asarray(v) for k, v in prm.items()},
             **{k: np.asarray(v) for k, v in r.items()})


if __name__ == "__main__":
    main()
    refkernel_ops()
    registration_cases()
