"""End-to-end parity curve of the GPU solver against the CPU restatement of
NestaUp::launch (src/processes/nesta/NestaUp.cpp:442-910), iteration by
iteration, at the headline workload (256x256x20 frames, 12 coils, R = 8,
lambda_i = 0.01, mu_f = 1e-3, one continuation step, no stopping test).

With maxIntIter = 1 and stoptest = 0 the k-th iterate of a long run equals the
output of a run with maxIter = k, so the restatement runs once with snapshots
and the GPU runs once per k.  For every k the script prints

    NRMSE(gpu, f32)   distance of the GPU result from the FP32 restatement
    NRMSE(f32, f64)   distance of the FP32 restatement from the FP64 oracle
    NRMSE(gpu, f64)   distance of the GPU result from the FP64 oracle

for the plain FP32 solver and, with --mixed, for the mixed-precision form.
Both FP32 implementations drift from FP64 at the same rate: the
100-iteration trajectory amplifies any ~1e-7 perturbation, so two FP32
implementations with different operation orders agree to 1e-4 only over the
first iterations.  tests/test_nesta_gpu.py asserts the 1e-4 bar over the range
this curve shows.

Needs a GPU.  Usage:
    python tests/parity_curve.py [--iters 1,2,5,10,20,50,100] [--size 256,256,20,12,8]
                                 [--mixed] [--json out.json]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import opencliper_gb300 as g  # noqa: E402
from opencliper_gb300 import synth  # noqa: E402
from oracle import drand48  # noqa: E402
from oracle import nesta_ref as R  # noqa: E402

PRM = dict(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, stoptest=0, miniter=7, tolVar=3e-4)


def gpu_run(ctx, dev, shape, k: int, mixed: bool) -> np.ndarray:
    F, C, H, W = shape
    x = ctx.empty((F, H, W), np.complex64)
    ctx.seed48(drand48.state_to_seed16v(drand48.DEFAULT_STATE))
    prm = g.nesta_params(**PRM, maxIter=k)
    prob = g.Problem(ctx, *dev)
    if mixed:
        b = g.Batch(ctx, [prob], prm, [x], precision=g.PRECISION_MIXED)
        b.launch()
        st = b.stats(0)
        b.close()
    else:
        st = prob.run(prm, x)
    prob.close()
    if st["status"] != 0 or st["inner_iters"] != k:
        raise RuntimeError(f"GPU run k={k}: status {st['status']}, {st['inner_iters']} iterations")
    return x.get()


def curve(size, iters, mixed: bool):
    W, H, F, C, Rr = size
    p = synth.make_problem(W, H, F, C, Rr, seed=0)
    kmax = max(iters)
    t0 = time.perf_counter()
    r32 = R.nesta(p.y, p.S, p.mask, R.NestaParams(**PRM, maxIter=kmax), "f32", snapshots=set(iters))
    r64 = R.nesta(p.y, p.S, p.mask, R.NestaParams(**PRM, maxIter=kmax), "f64", snapshots=set(iters))
    t_oracle = time.perf_counter() - t0
    rows = []
    with g.Context(0) as ctx:
        dev = (ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask))
        for k in iters:
            x32, x64 = r32.stats["snapshots"][k], r64.stats["snapshots"][k]
            row = dict(k=k, f32_f64=R.nrmse(x32, x64))
            xg = gpu_run(ctx, dev, p.y.shape, k, False)
            row.update(gpu_f32=R.nrmse(xg, x32), gpu_f64=R.nrmse(xg, x64))
            if mixed:
                xm = gpu_run(ctx, dev, p.y.shape, k, True)
                row.update(mixed_f32=R.nrmse(xm, x32), mixed_f64=R.nrmse(xm, x64))
            rows.append(row)
    return rows, t_oracle


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--iters", default="1,2,5,10,20,50,100")
    ap.add_argument("--size", default="256,256,20,12,8", help="W,H,F,C,R")
    ap.add_argument("--mixed", action="store_true")
    ap.add_argument("--json", default=None)
    a = ap.parse_args(argv)
    iters = sorted({int(v) for v in a.iters.split(",")})
    size = tuple(int(v) for v in a.size.split(","))
    rows, t_oracle = curve(size, iters, a.mixed)
    cols = ["k", "gpu_f32", "f32_f64", "gpu_f64"] + (["mixed_f32", "mixed_f64"] if a.mixed else [])
    names = {"k": "iterations", "gpu_f32": "NRMSE(gpu, f32)", "f32_f64": "NRMSE(f32, f64)",
             "gpu_f64": "NRMSE(gpu, f64)", "mixed_f32": "NRMSE(mixed, f32)", "mixed_f64": "NRMSE(mixed, f64)"}
    print(f"workload W,H,F,C,R = {size}; oracle time {t_oracle:.1f} s")
    print("| " + " | ".join(names[c] for c in cols) + " |")
    print("|" + "---|" * len(cols))
    for r in rows:
        print("| " + " | ".join(str(r[c]) if c == "k" else f"{r[c]:.2e}" for c in cols) + " |")
    if a.json:
        with open(a.json, "w") as fh:
            json.dump(dict(size=size, rows=rows), fh, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
