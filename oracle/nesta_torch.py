"""Restatement of NestaUp::launch with torch tensors -- test infrastructure
(oracle): the FP64 oracle for large workloads, and an FP32 variant that
measures how far FP32 rounding alone moves the result at a given size.

The same algorithm as oracle/nesta_ref.py's precision="f64" mode, statement for
statement, written with torch so that it runs on a CUDA device (torch.fft,
i.e. cuFFT, in double precision) as well as on the CPU.  It exists for the
large workloads (384x384 x 30 frames x 16 coils, the uneven batch) where the
numpy FP64 oracle takes minutes per reconstruction; tests/test_oracle.py pins
it to nesta_ref's FP64 mode on small problems.  With dtype complex64 the
arrays are FP32 (scalars stay Python floats): an FP32 implementation whose
distance from the FP64 result is the FP32 noise floor of that workload.  Only
the plain (no motion compensation) form is restated here.

Citations are to src/processes/nesta/NestaUp.cpp of the reference.
"""
from __future__ import annotations

import numpy as np

from . import drand48
from .nesta_ref import NestaParams


def _ttv(x, forward: bool):
    """operator_tTV / operator_tTVadj (temporalTV.cl:49-107)."""
    import torch
    if forward:
        return x - torch.roll(x, 1, dims=0)
    return torch.roll(x, -1, dims=0) - x


def _nrm2sq(v) -> float:
    return float((v.real * v.real + v.imag * v.imag).sum())


def _normest(F: int, H: int, W: int, rand_state: int, dev, cdt=None):
    """myNormest (NestaUp.cpp:291-439) in double precision: the all-ones start
    gives U x = 0, so the first pass restarts from drand48 values."""
    import torch
    cdt = cdt or torch.complex128
    tol, maxiter = 1e-3, 100
    x = torch.ones((F, H, W), dtype=cdt, device=dev)
    e = float(np.sqrt(float(F * H * W)))
    x = x / e
    e0 = 0.0
    cnt = 0
    state = rand_state
    while abs(e - e0) > tol * e and cnt < maxiter:
        e0 = e
        Sx = _ttv(x, True)
        nnz = float((Sx.real.abs() + Sx.imag.abs()).sum())
        if nnz == 0:
            vals, state = drand48.lcg_sequence(F * H * W, state)
            # complexType(drand48(), 0) stored as float in the reference
            Sx = torch.from_numpy(vals.astype(np.float32).astype(np.float64).reshape(F, H, W)).to(dev)
            Sx = torch.complex(Sx, torch.zeros_like(Sx)).to(cdt)
        e = float(np.sqrt(_nrm2sq(Sx)))
        x = _ttv(Sx, False)
        x = x / float(np.sqrt(_nrm2sq(x)))
        cnt += 1
    return e, cnt, state


def nesta_f64(y: np.ndarray, S: np.ndarray, mask: np.ndarray, prm: NestaParams,
              rand_state: int = drand48.DEFAULT_STATE, device: str = "cpu", fp32: bool = False,
              fp64_state: tuple = ()) -> tuple[np.ndarray, dict]:
    """FP64 NESTA of y [F][C][H][W], S [C][H][W], pixel mask [F][H][W]; returns
    (image [F][H][W], stats).  Inputs may be numpy arrays or torch tensors (a
    tensor already on `device` is used in place).  fp32=True runs the same
    statements on complex64 arrays; with it, fp64_state may name iteration
    state kept in complex128 all the same: "w" (the weighted gradient sum of
    NestaUp.cpp:837-840) and "x" (x_k, y_k, z_k and x_ref)."""
    import torch
    dev = torch.device(device)
    cdt = torch.complex64 if fp32 else torch.complex128
    wdt = torch.complex128 if "w" in fp64_state else cdt
    xdt = torch.complex128 if "x" in fp64_state else cdt

    def T(a, dt):
        t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
        return t.to(dev).to(dt)

    y = T(y, cdt)
    S = T(S, cdt)
    keep = T(mask, torch.uint8) != 0
    F, Cn, H, W = y.shape
    N = H * W
    Sc = S.conj()

    def A(x):   # operatorA (162-190): mask(FFT_fwd(S x))
        k = torch.fft.fft2(x[:, None] * S[None])
        return torch.where(keep[:, None], k, torch.zeros((), dtype=k.dtype, device=dev))

    def At(k):  # operatorAt (117-151): sum_c conj(S_c) IFFT(k_c), no mask
        return (torch.fft.ifft2(k) * Sc[None]).sum(dim=1)

    sqrtN = float(np.sqrt(float(N)))
    xref = At(y * sqrtN)                       # x0 (465-486)
    Ux0 = _ttv(xref, True)
    maxX = float(xref.abs().max())             # (521-568)
    maxUX = float(Ux0.abs().max())
    miniter = int(prm.miniter)
    lam = prm.lambda_i * maxX
    muf = prm.mu_f * maxX
    mu0 = 0.9 * maxUX
    normU, ne_iters, new_state = _normest(F, H, W, rand_state, dev, cdt)
    if lam / prm.La > mu0:
        mu0 = lam / prm.La
    gamma = (muf / mu0) ** (1.0 / prm.maxIntIter)
    mu = mu0
    gammat = (prm.tolVar / 0.1) ** (1.0 / prm.maxIntIter)
    tolVar = 0.1
    fmean = np.zeros(max(miniter, 1), np.float64)
    inv_sqrtN = 1.0 / np.sqrt(float(N))
    fx = qp = 0.0
    iters = 0
    xref = xref.to(xdt)
    for nl in range(1, prm.maxIntIter + 1):
        mu *= gamma
        tolVar *= gammat
        w = torch.zeros(xref.shape, dtype=wdt, device=dev)
        xk = xref.clone()
        Lmu = normU / mu
        if miniter > 0:
            fmean[miniter - 1] = float(np.float32(9223372036854775807))
        Lmu = lam * Lmu + prm.La
        Lmu1 = 1.0 / Lmu
        qpDone = False
        k = 0
        while k < prm.maxIter:
            xc = xk.to(cdt)
            d = _ttv(xc, True)                                   # operatorU (669)
            u = d / torch.clamp(d.abs(), min=mu)                 # VectorNormalization (680-683)
            normUk = np.sqrt(_nrm2sq(u))                         # Scnrm2 (686)
            fxdot = float((u.conj() * d).real.sum())             # Cdotc real part (691)
            Df = -_ttv(u, False)                                 # operatorUt + Cscal(-1) (696-704)
            res = A(xc) * inv_sqrtN - y                          # (710-727)
            l2 = _nrm2sq(res)                                    # (738-746)
            Df = Df * lam + At(res * sqrtN)                      # (749-772)
            yk = xk - Lmu1 * Df.to(xdt)                          # (777-786)
            l1term = fxdot - mu / 2.0 * normUk ** 2              # (797-798)
            fx = 0.5 * l2 + lam * l1term
            if prm.stoptest == 1:                                # (799-824)
                brk = False
                if k >= miniter:
                    fm = sum(fmean[miniter - ne - 1] for ne in range(miniter)) / miniter
                    qp = (fm - fx) / fm
                    if qp <= tolVar:
                        if qpDone:
                            k = prm.maxIter
                        qpDone = True
                        brk = True
                else:
                    qp = fmean[miniter - 1]
                if not brk:
                    fmean[(miniter - 1) - ((k + 1) % miniter)] = fx
            apk = 0.5 * (k + 1.0)                                # (829-831)
            tauk = 2.0 / (k + 3.0)
            w = w + apk * Df.to(wdt)                             # (837-840)
            zk = xref - (Lmu1 * w).to(xdt)                       # (843-852)
            xk = tauk * zk + (1.0 - tauk) * yk                   # (858-875)
            iters += 1
            k += 1
        xref = xk                                                # (889)
    stats = dict(normU=normU, normest_iters=ne_iters, maxX=maxX, maxUX=maxUX, lambda_=lam, muf=muf, mu0=mu0,
                 mu_final=mu, tolVar_final=tolVar, fx_final=fx, qp_final=qp, inner_iters=iters, rand_state=new_state)
    return xref.to(cdt).cpu().numpy(), stats
