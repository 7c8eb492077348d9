"""Motion-compensated sparsity operator of NESTA -- TEST INFRASTRUCTURE
(oracle): restatement of MotionCompensation / AdjointMotionCompensation
(src/processes/MotionCompensation.cpp:57-78, AdjointMotionCompensation.cpp:
59-86) and their kernels (src/kernels/optimizer.cl:832-937 interpolator /
adjointInterpolator, src/kernels/initialize.cl:55-80 initZeroRect /
copyDataGPU).  Pinned bit for bit against those kernels compiled for the host
(oracle/refkernels.py).

Layouts (as ArgumentsMotionCompensation holds them, GroupwiseRegistration.hpp:
95-100): xmesh = original mesh [2][W][H] int32, xn = deformed mesh [2][F][H][W]
float32, both 1-based (index 0 horizontal = column, 1 vertical = row); bb = the
1-based bounding box (bound_box).  The rectangle covers rows r1 and columns r2
(Interpolator.cpp:63-87, margins H/40 and W/40 in integer division)."""
from __future__ import annotations

import numpy as np


def rect(W: int, H: int, bb) -> tuple[np.ndarray, np.ndarray]:
    m0, m1 = H // 40, W // 40
    l1 = (bb[3] + m0 + 1) - (bb[1] - m0 - 1) + 1
    l2 = (bb[2] + m1 + 1) - (bb[0] - m1 - 1) + 1
    r1 = np.array([(bb[1] - m0 - 1) + i - 1 for i in range(l1)], np.int64)
    r2 = np.array([(bb[0] - m1 - 1) + j - 1 for j in range(l2)], np.int64)
    return r1, r2


def _geometry(shape, xn, xmesh, bb):
    F, H, W = shape
    r1, r2 = rect(W, H, bb)
    # work-items in the harness order: frame outer, then column index j, then row index i
    k, j, i = np.meshgrid(np.arange(F), np.arange(len(r2)), np.arange(len(r1)), indexing="ij")
    k, j, i = k.ravel(), j.ravel(), i.ravel()
    R1, R2 = r1[i], r2[j]
    hor = xmesh[0, R2, R1].astype(np.int64) - 1
    ver = xmesh[1, R2, R1].astype(np.int64) - 1
    one = np.float32(1)
    nhor = xn[0, k, R1, R2].astype(np.float32) - one
    nver = xn[1, k, R1, R2].astype(np.float32) - one
    prehor = np.floor(nhor).astype(np.int64)
    prever = np.floor(nver).astype(np.int64)
    return k, R1, R2, hor, ver, nhor, nver, prehor, prever


def warp(x: np.ndarray, xn, xmesh, bb) -> np.ndarray:
    """MotionCompensation: out = x, then out[hor, ver] = bilinear x at (nhor, nver)."""
    x = np.asarray(x)
    out = x.copy()
    k, R1, R2, hor, ver, nhor, nver, ph, pv = _geometry(x.shape, xn, xmesh, bb)
    qh, qv = ph + 1, pv + 1
    a, b = qh.astype(np.float32) - nhor, nhor - ph.astype(np.float32)
    c, d = qv.astype(np.float32) - nver, nver - pv.astype(np.float32)
    if x.dtype == np.complex64:
        i1, i2, i3, i4 = x[k, pv, ph], x[k, pv, qh], x[k, qv, ph], x[k, qv, qh]
        aux1 = (a * i1.real + b * i2.real) + 1j * (a * i1.imag + b * i2.imag)
        aux2 = (a * i3.real + b * i4.real) + 1j * (a * i3.imag + b * i4.imag)
        val = (c * aux1.real + d * aux2.real) + 1j * (c * aux1.imag + d * aux2.imag)
        out[k, ver, hor] = val.astype(np.complex64)
    else:
        a, b, c, d = (v.astype(np.float64) for v in (a, b, c, d))
        aux1 = a * x[k, pv, ph] + b * x[k, pv, qh]
        aux2 = a * x[k, qv, ph] + b * x[k, qv, qh]
        out[k, ver, hor] = c * aux1 + d * aux2
    return out


def warp_adjoint(g: np.ndarray, xn, xmesh, bb) -> np.ndarray:
    """AdjointMotionCompensation: out = g, zero the rectangle, then scatter each
    rectangle value back with its bilinear weights."""
    g = np.asarray(g)
    F, H, W = g.shape
    r1, r2 = rect(W, H, bb)
    out = g.copy()
    out[:, r1[:, None], r2[None, :]] = 0
    k, R1, R2, hor, ver, nhor, nver, ph, pv = _geometry(g.shape, xn, xmesh, bb)
    rt = np.float32 if g.dtype == np.complex64 else np.float64
    Wvv = (nver - pv.astype(np.float32)).astype(rt)
    Whh = (nhor - ph.astype(np.float32)).astype(rt)
    one = rt(1)
    i0 = g[k, ver, hor]
    flat = lambda kk, vv, hh: (kk * H + vv) * W + hh
    tgt = [flat(k, pv, ph), flat(k, pv, ph + 1), flat(k, pv + 1, ph), flat(k, pv + 1, ph + 1)]
    idx = np.stack(tgt, axis=1).ravel()  # per work-item its four targets, work-items in order
    re, im = out.real.ravel().copy(), out.imag.ravel().copy()
    for part, acc in ((i0.real.astype(rt), re), (i0.imag.astype(rt), im)):
        w = np.stack([part * (one - Whh) * (one - Wvv), part * Whh * (one - Wvv), part * (one - Whh) * Wvv,
                      part * Whh * Wvv], axis=1).ravel()
        np.add.at(acc, idx, w)  # unbuffered, in index-array order
    return (re + 1j * im).reshape(F, H, W).astype(g.dtype)
