"""CPU restatement of OpenCLIPER's tTV-NESTA path -- test infrastructure.

Every function follows the reference source it cites (paths relative to the
reference project).  `precision="f32"` mirrors the reference's arithmetic
types (complex64 data, float host scalars, double where the reference calls
std::pow/sqrt on doubles); `precision="f64"` runs the same algorithm entirely in
double precision and is the FP64 oracle for error reporting.

FFT conventions are clFFT's (FFT.cpp:374-525): forward unscaled, backward
scaled by 1/N, no fftshift -- numpy's fft2/ifft2 defaults.  CLBlast's BLAS-1
calls are restated from their definitions: nrm2 = sqrt(sum |z|^2),
dotc(a, b) = sum conj(a) b, asum = sum |Re| + |Im|.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np
import scipy.fft as sfft

from . import drand48

LONG_MAX_F32 = np.float32(9223372036854775807)  # float(LONG_MAX), NestaUp.cpp:645


class _P:
    """Scalar/array types of one precision mode."""

    def __init__(self, precision: str):
        if precision not in ("f32", "f64"):
            raise ValueError(precision)
        self.f32 = precision == "f32"
        self.r = np.float32 if self.f32 else np.float64
        self.c = np.complex64 if self.f32 else np.complex128

    def s(self, v):
        """host 'float' scalar of the reference (float32 in f32 mode)."""
        return self.r(v)


def _workers() -> int:
    return int(os.environ.get("ORACLE_WORKERS", os.cpu_count() or 1))


# ---------------------------------------------------------------------------
# Operators
# ---------------------------------------------------------------------------
def fft2(a: np.ndarray, forward: bool) -> np.ndarray:
    """FFT process, dim=-1 (FFT.cpp:116-201): 2-D over the last two axes."""
    if forward:
        return sfft.fft2(a, axes=(-2, -1), workers=_workers())
    return sfft.ifft2(a, axes=(-2, -1), workers=_workers())


def ttv(x: np.ndarray, forward: bool) -> np.ndarray:
    """TemporalTV: operator_tTV temporalTV.cl:49-76 (out[f] = in[f] - in[f-1],
    frame 0 uses frame F-1) and operator_tTVadj temporalTV.cl:78-107
    (out[f] = in[f+1] - in[f], frame F-1 uses frame 0)."""
    if forward:
        return x - np.roll(x, 1, axis=0)
    return np.roll(x, -1, axis=0) - x


def normalize(d: np.ndarray, mu) -> np.ndarray:
    """vectorNormalization.cl:42-56: out = in / fmax(mu, length(in))."""
    m = np.maximum(np.asarray(mu, d.real.dtype), np.abs(d))
    return d / m


def sensmul(x: np.ndarray, S: np.ndarray, conjugate: bool) -> np.ndarray:
    """complexElementProd.cl:42-76: out[f][c] = in[f](or in[f][c]) * S[c] or * conj(S[c])."""
    s = np.conj(S) if conjugate else S
    if x.ndim == 3:
        return x[:, None, :, :] * s[None]
    return x * s[None]


def coilsum(k: np.ndarray) -> np.ndarray:
    """xImageSum.cl:42-61: sum over coils in order c = 0..C-1."""
    acc = k[:, 0].copy()
    for c in range(1, k.shape[1]):
        acc += k[:, c]
    return acc


def apply_mask(k: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """applyMask.cl:5-40: zero where the pixel mask is 0 (mask [F][H][W])."""
    return np.where(mask[:, None, :, :] == 0, np.zeros((), k.dtype), k)


def rowmask_to_pixelmask(rowmask: np.ndarray, W: int) -> np.ndarray:
    """SamplingMasksData::rowmask2pixelmask (SamplingMasksData.cpp:389-441):
    1 -> 255 across the row, 0 -> 0, anything else is an error."""
    if np.any((rowmask != 0) & (rowmask != 1)):
        raise ValueError("sampling mask data element must be 0 or 1")
    return np.repeat((rowmask.astype(np.uint8) * 255)[:, :, None], W, axis=2)


def complex_abs(x: np.ndarray) -> np.ndarray:
    """complexAbs.cl:43-70: (sqrt(re^2 + im^2), 0)."""
    return np.abs(x).astype(x.real.dtype).astype(x.dtype)


def complex_abs2(x: np.ndarray) -> np.ndarray:
    """complexAbsPow2.cl:43-71: (re^2 + im^2, 0)."""
    return (x.real * x.real + x.imag * x.imag).astype(x.dtype)


def operator_A(x, S, mask):
    """NestaUp::operatorA (NestaUp.cpp:162-190): mask(FFT_fwd(S x))."""
    return apply_mask(fft2(sensmul(x, S, False), True), mask)


def operator_At(k, S):
    """NestaUp::operatorAt (NestaUp.cpp:117-151): sum_c conj(S_c) IFFT(k_c) (no mask)."""
    return coilsum(sensmul(fft2(k, False), S, True))


def encode(x, S, mask):
    """operatorA followed by the 1/sqrt(N) Cscal of NestaUp.cpp:712-718."""
    N = x.shape[-1] * x.shape[-2]
    f = np.float32(1.0 / np.sqrt(np.float64(N)))  # double expression stored in a float
    return operator_A(x, S, mask) * f


def encode_adjoint(k, S):
    """sqrt(N) Cscal (NestaUp.cpp:749-753) then operatorAt."""
    N = k.shape[-1] * k.shape[-2]
    return operator_At(k * np.sqrt(np.float32(N)), S)


def simple_recon(y, S):
    """SimpleMRIRecon::launch (SimpleMRIRecon.cpp:80-101): IFFT, * conj(S), coil sum."""
    return coilsum(sensmul(fft2(y, False), S, True))


def rss(k: np.ndarray) -> np.ndarray:
    """RSoS::launch + rss.cl:43-74 on KData [F][C][H][W]: (sqrt(sum_c |k_c|^2), 0),
    the sum accumulated in the data's real type in coil order."""
    F, Cn, H, W = k.shape
    acc = np.zeros((F, H, W), k.real.dtype)
    for c in range(Cn):
        kc = k[:, c]
        acc = acc + (kc.real * kc.real + kc.imag * kc.imag)
    return np.sqrt(acc).astype(k.dtype)


def simple_recon_sos(y: np.ndarray) -> np.ndarray:
    """SimpleMRIReconSOS::launch (SimpleMRIReconSOS.cpp:65-118): backward FFT of
    every coil image, then the root sum of squares over coils."""
    return rss(fft2(y, False))


# ---------------------------------------------------------------------------
# Power method (myNormest, NestaUp.cpp:291-439)
# ---------------------------------------------------------------------------
def normest(F: int, H: int, W: int, precision: str = "f32", rand_state: int = drand48.DEFAULT_STATE,
            use_libc: bool = False, U=None, Ut=None):
    """Returns (e, iterations, new drand48 state).

    The loop test uses the float overload of abs: CLapp.hpp:54 includes
    <stdlib.h>, whose C++ wrapper brings std::abs(float) into the global
    namespace that NestaUp.cpp's unqualified abs() call resolves against.
    U / Ut: the sparsity operator and its adjoint (default: temporal TV and its
    adjoint kernel; with motion compensation, NestaUp::operatorU/Ut)."""
    U = U or (lambda v: ttv(v, True))
    Ut = Ut or (lambda v: ttv(v, False))
    P = _P(precision)
    n = P.s(np.float32(H * W * F)) if P.f32 else float(H * W * F)
    tol = P.s(1e-3)
    maxiter = 100
    x = np.ones((F, H, W), P.c)
    e = P.s(np.sqrt(np.sum(np.abs(x) ** 2, dtype=np.float64)))
    x = x * P.s(1 / e)
    e0 = P.s(0)
    cnt = 0
    state = rand_state
    while abs(e - e0) > tol * e and cnt < maxiter:
        e0 = e
        Sx = U(x)
        nnz = np.sum(np.abs(Sx.real) + np.abs(Sx.imag))
        if nnz == 0:
            gen = drand48.libc_sequence if use_libc else drand48.lcg_sequence
            vals, state = gen(F * H * W, state)
            Sx = vals.astype(np.float32).reshape(F, H, W).astype(P.c)  # complexType(drand48(), 0)
        e = P.s(np.sqrt(np.sum(np.abs(Sx) ** 2, dtype=np.float64)))
        x = Ut(Sx)  # operatorUt: tTVadj then copy / adjoint motion compensation (no negation here)
        nx = P.s(np.sqrt(np.sum(np.abs(x) ** 2, dtype=np.float64)))
        x = x * P.s(1 / nx)
        cnt += 1
    return e, cnt, state


# ---------------------------------------------------------------------------
# NESTA (NestaUp::launch, NestaUp.cpp:442-910)
# ---------------------------------------------------------------------------
@dataclass
class NestaParams:
    """NestaUp::LaunchParameters (NestaUp.hpp:67-83)."""
    lambda_i: float = 1e-2
    mu_f: float = 3e-4
    La: float = 1.0
    maxIntIter: int = 4
    tolVar: float = 3e-4
    verbose: int = 1
    maxIter: int = 100
    stoptest: int = 1
    miniter: int = 7


@dataclass
class NestaResult:
    x: np.ndarray
    stats: dict = field(default_factory=dict)


def _nrm2sq(v: np.ndarray) -> float:
    return float(np.sum(v.real.astype(np.float64) ** 2 + v.imag.astype(np.float64) ** 2))


def nesta(y: np.ndarray, S: np.ndarray, mask: np.ndarray, prm: NestaParams, precision: str = "f32",
          rand_state: int = drand48.DEFAULT_STATE, record: bool = False, timings: dict | None = None,
          mc=None, x_init: np.ndarray | None = None, snapshots=None) -> NestaResult:
    """y: KData [F][C][H][W]; S: [C][H][W]; mask: pixel mask [F][H][W] (uint8).
    `timings`, when given, receives wall-clock marks: 'setup' (seconds until the
    first inner iteration) and 'iters' (seconds of each inner iteration).
    `mc` = (xn, xmesh, bb) runs the motion-compensated form (argsMC != nullptr):
    the sparsity operator becomes U = tTV(M x), Ut = M^T tTVadj (NestaUp.cpp:
    201-278), and the solve starts from `x_init` (the output XData's current
    image) instead of E^H y (NestaUp.cpp:483-486).
    `snapshots`: inner-iteration counts k at which x_k (the iterate after k
    inner iterations, counted over all outer loops) is copied into
    stats["snapshots"][k]; with maxIntIter = 1 and stoptest = 0 it equals the
    output of a run with maxIter = k."""
    import time as _time
    _t0 = _time.perf_counter()
    P = _P(precision)
    F, Cn, H, W = y.shape
    N = H * W
    y = y.astype(P.c)
    S = S.astype(P.c)
    s = P.s
    # y' = copy(y) * sqrt(float(N))   (NestaUp.cpp:465-481)
    sqrtN = s(np.sqrt(np.float32(N))) if P.f32 else np.sqrt(float(N))
    yp = y * sqrtN
    if mc is not None:
        from oracle import motion
        xn_, xm_, bb_ = mc

        def U(v):
            return ttv(motion.warp(v, xn_, xm_, bb_), True)

        def Ut(v):
            return motion.warp_adjoint(ttv(v, False), xn_, xm_, bb_)
        xref = np.asarray(x_init).astype(P.c)
    else:
        def U(v):
            return ttv(v, True)

        def Ut(v):
            return ttv(v, False)
        # x0 = operatorAt(y')  (NestaUp.cpp:484-486)
        xref = operator_At(yp, S).astype(P.c)
    Ux0 = U(xref)
    # maxima (NestaUp.cpp:521-568)
    maxX = s(np.max(np.abs(xref)))
    maxUX = s(np.max(np.abs(Ux0)))
    miniter = int(prm.miniter)
    lam = s(s(prm.lambda_i) * maxX)
    muf = s(s(prm.mu_f) * maxX)
    mu0 = s(0.9 * float(maxUX))
    normU, ne_iters, new_state = normest(F, H, W, precision, rand_state, U=U, Ut=Ut)
    muL = s(lam / s(prm.La))
    if muL > mu0:
        mu0 = muL
    gamma = s(np.power(np.float64(muf / mu0), 1.0 / prm.maxIntIter))
    mu = mu0
    gammat = s(np.power(np.float64(prm.tolVar) / 0.1, 1.0 / prm.maxIntIter))
    tolVar = s(0.1)
    fmean = np.zeros(max(miniter, 1), P.r)
    inv_sqrtN = s(1.0 / np.sqrt(np.float64(N)))  # NestaUp.cpp:712: double expression stored in a float
    fx = s(0)
    qp = s(0)
    iters = 0
    hist = []
    snaps = {}
    if timings is not None:
        timings["setup"] = _time.perf_counter() - _t0
        timings["iters"] = []
    for nl in range(1, prm.maxIntIter + 1):
        mu = s(mu * gamma)
        tolVar = s(tolVar * gammat)
        w = np.zeros_like(xref)
        xk = xref.copy()
        Ak = s(0)
        Lmu = s(normU / mu)
        if miniter > 0:
            fmean[miniter - 1] = LONG_MAX_F32 if P.f32 else float(np.float32(9223372036854775807))
        Lmu = s(lam * Lmu + s(prm.La))
        Lmu1 = s(1 / Lmu)
        qpDone = False
        k = 0
        while k < prm.maxIter:
            d = U(xk)                               # operatorU (669)
            u = normalize(d, mu)                    # VectorNormalization (680-683)
            normUk = s(np.sqrt(_nrm2sq(u)))         # Scnrm2 (686)
            fxdot = s(np.sum((np.conj(u) * d).real, dtype=np.float64))  # Cdotc real part (691)
            Df = -Ut(u)                             # operatorUt + Cscal(-1) (696-704)
            res = operator_A(xk, S, mask) * inv_sqrtN - y  # operatorA, Cscal(1/sqrt N), Caxpy(-1) (710-727)
            l2 = s(_nrm2sq(res))                    # ComplexAbsPow2 + Scsum (738-746)
            Ares = operator_At(res * sqrtN, S)      # Cscal(sqrt N) + operatorAt (749-756)
            Df = Df * lam + Ares                    # Cscal(lambda), Caxpy(1) (759-772)
            yk = xk + (-Lmu1) * Df                  # Ccopy + Caxpy(-Lmu1) (777-786)
            # objective and stopping test (797-824)
            l1term = s(float(fxdot) - float(s(mu / s(2.0))) * float(normUk) ** 2)
            fx = s(s(0.5) * l2 + lam * l1term)
            if prm.stoptest == 1:
                brk = False
                if k >= miniter:
                    fm = s(0)
                    for ne in range(miniter):
                        fm = s(fm + fmean[miniter - ne - 1])
                    fm = s(fm / s(miniter))
                    qp = s((fm - fx) / fm)
                    if qp <= tolVar:
                        if qpDone:
                            k = prm.maxIter
                        qpDone = True
                        brk = True
                else:
                    qp = fmean[miniter - 1]
                if not brk:
                    fmean[(miniter - 1) - ((k + 1) % miniter)] = fx
            apk = s(s(0.5) * (s(k) + s(1.0)))       # (829-831)
            Ak = s(Ak + apk)
            tauk = s(s(2.0) / (s(k) + s(3.0)))
            w = w + apk * Df                        # Caxpy(apk) (837-840)
            zk = xref + (-Lmu1) * w                 # Ccopy + Caxpy(-Lmu1) (843-852)
            xk = tauk * zk + (s(1.0) - tauk) * yk   # Ccopy, Cscal(tauk), Caxpy(1-tauk) (858-875)
            xk = xk.astype(P.c)
            w = w.astype(P.c)
            iters += 1
            if timings is not None:
                _t1 = _time.perf_counter()
                timings["iters"].append(_t1 - _t0 - timings["setup"] - sum(timings["iters"]))
            if record:
                hist.append(float(fx))
            if snapshots is not None and iters in snapshots:
                snaps[iters] = xk.copy()
            k += 1
        xref = xk.copy()                            # (889)
    stats = dict(normU=float(normU), normest_iters=ne_iters, maxX=float(maxX), maxUX=float(maxUX),
                 lambda_=float(lam), muf=float(muf), mu0=float(mu0), mu_final=float(mu),
                 tolVar_final=float(tolVar), fx_final=float(fx), qp_final=float(qp), inner_iters=iters,
                 rand_state=new_state)
    if record:
        stats["fx_hist"] = hist
    if snapshots is not None:
        stats["snapshots"] = snaps
    return NestaResult(xref, stats)


def nrmse(x: np.ndarray, ref: np.ndarray) -> float:
    """||x - ref||_2 / ||ref||_2 over all frames."""
    ref64 = ref.astype(np.complex128)
    return float(np.linalg.norm((x.astype(np.complex128) - ref64).ravel()) / np.linalg.norm(ref64.ravel()))
