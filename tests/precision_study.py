"""What 16-bit storage of the inputs does to the final image, against the
metric's NRMSE <= 1e-3 gate: the NESTA solve of the headline workload
(256x256x20 frames, 12 coils, R = 8, lambda_i 0.01, mu_f 1e-3, 100 iterations)
run in FP64 on inputs rounded to 16 bits, compared with the FP64 solve of the
unrounded inputs, next to the FP32 noise floor (the same solve on complex64
arrays).  The rounding schemes:

    fp16 / bf16, one power-of-two scale per coil     (k-space y)
    fp16 / bf16, one scale per (frame, row, coil)    (k-space y: the dynamic
                                                      range of k-space lives
                                                      along the phase-encode rows)
    fp16, one scale per coil                         (coil maps S)

A scheme whose error stays under the gate with room beside the FP32 floor
could store that operand in 16 bits; each solve runs the FP64 restatement
oracle/nesta_torch.py (torch; a CUDA device when available).  A second table
keeps iteration state in FP64 inside the FP32 solve (the weighted gradient
sum w, the iterate x, both): if the FP32 floor came from accumulating w or x
it would drop there.

    python tests/precision_study.py [--size 256,256,20,12,8] [--iters 100] [--device cuda]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from opencliper_gb300 import synth  # noqa: E402
from oracle import nesta_ref as R  # noqa: E402
from oracle import nesta_torch as RT  # noqa: E402


def _round16(a: np.ndarray, kind: str, scale_axes: tuple) -> np.ndarray:
    """Round the real and imaginary parts of complex `a` to fp16 or bf16 after
    a power-of-two scale per slice (the max over scale_axes brought to 2^14),
    then undo the scale."""
    import torch
    re, im = np.real(a).astype(np.float32), np.imag(a).astype(np.float32)
    mx = np.maximum(np.abs(re).max(axis=scale_axes, keepdims=True), np.abs(im).max(axis=scale_axes, keepdims=True))
    e = np.where(mx > 0, np.floor(np.log2(np.where(mx > 0, mx, 1.0))), 0.0)
    sig = np.exp2(13.0 - e).astype(np.float32)
    dt = torch.float16 if kind == "fp16" else torch.bfloat16

    def r(v):
        return torch.from_numpy(np.ascontiguousarray(v * sig)).to(dt).to(torch.float32).numpy() / sig

    return (r(re) + 1j * r(im)).astype(np.complex64)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--size", default="256,256,20,12,8", help="W,H,F,C,R")
    ap.add_argument("--iters", type=int, default=100)
    ap.add_argument("--device", default=None)
    a = ap.parse_args(argv)
    import torch
    dev = a.device or ("cuda" if torch.cuda.is_available() else "cpu")
    W, H, F, C, Rr = (int(v) for v in a.size.split(","))
    p = synth.make_problem(W, H, F, C, Rr, seed=0)
    prm = R.NestaParams(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=a.iters, stoptest=0, miniter=7)
    ref, _ = RT.nesta_f64(p.y, p.S, p.mask, prm, device=dev)
    x32, _ = RT.nesta_f64(p.y, p.S, p.mask, prm, device=dev, fp32=True)
    print(f"workload W,H,F,C,R = {(W, H, F, C, Rr)}, {a.iters} iterations, device {dev}")
    print(f"| scheme | NRMSE vs FP64 |\n|---|---|\n| FP32 arrays (noise floor) | {R.nrmse(x32, ref):.2e} |")
    cases = [("y fp16, scale per coil", "y", "fp16", (0, 2, 3)),
             ("y bf16, scale per coil", "y", "bf16", (0, 2, 3)),
             ("y fp16, scale per (frame, row, coil)", "y", "fp16", (3,)),
             ("y bf16, scale per (frame, row, coil)", "y", "bf16", (3,)),
             ("S fp16, scale per coil", "S", "fp16", (1, 2))]
    for name, which, kind, axes in cases:
        y, S = p.y, p.S
        if which == "y":
            y = _round16(p.y, kind, axes)
        else:
            S = _round16(p.S, kind, axes)
        x, _ = RT.nesta_f64(y, S, p.mask, prm, device=dev)
        print(f"| {name} | {R.nrmse(x, ref):.2e} |")
    print("\n| FP32 solve with FP64 state | NRMSE vs FP64 |\n|---|---|")
    for state in ((), ("w",), ("x",), ("w", "x")):
        x, _ = RT.nesta_f64(p.y, p.S, p.mask, prm, device=dev, fp32=True, fp64_state=state)
        print(f"| {', '.join(state) or 'none'} | {R.nrmse(x, ref):.2e} |")
    return 0


if __name__ == "__main__":
    sys.exit(main())
