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


if __name__ == "__main__":
    main()
    refkernel_ops()
