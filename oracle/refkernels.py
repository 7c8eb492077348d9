"""The reference's own operator kernels, compiled for the host -- TEST
INFRASTRUCTURE (oracle).

build() compiles src/kernels/{hostKernelFunctions,temporalTV,
vectorNormalization,complexElementProd,xImageSum,applyMask,complexAbsPow2,
complexAbs,rss,initialize,optimizer}.cl from the reference tree, with the host shim in
oracle/refkernels/shim and the harness oracle/refkernels/harness.cpp, into
oracle/_ref/librefkernels.so.  The reference tree is only read when present
(oracle.reference_root()); elsewhere the library is simply unavailable and
the tests that need it skip.  The functions below run the
kernels on numpy arrays in the reference layouts.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref" / "librefkernels.so"
from oracle import reference_root as _reference_root

_ROOT = _reference_root()
SOURCES = ["hostKernelFunctions.cl", "temporalTV.cl", "vectorNormalization.cl", "complexElementProd.cl",
           "xImageSum.cl", "applyMask.cl", "complexAbsPow2.cl", "complexAbs.cl", "rss.cl", "initialize.cl",
           "optimizer.cl", "creabspline.cl", "reductions.cl"]


def build(force: bool = False) -> Path | None:
    if _ROOT is None:
        return OUT if OUT.exists() else None
    kdir = _ROOT / "src" / "kernels"
    if not all((kdir / s).exists() for s in SOURCES):
        return OUT if OUT.exists() else None
    deps = [HERE / "refkernels" / "harness.cpp", HERE / "refkernels" / "shim" / "OpenCLIPER" / "kernels" /
            "hostKernelFunctions.h", HERE / "refkernels" / "registration_host.hpp"] + [kdir / s for s in SOURCES]
    if OUT.exists() and not force and all(d.stat().st_mtime <= OUT.stat().st_mtime for d in deps):
        return OUT
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        return None
    OUT.parent.mkdir(exist_ok=True)
    subprocess.run([cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-w", "-I", str(HERE / "refkernels" / "shim"),
                    "-I", str(kdir), str(HERE / "refkernels" / "harness.cpp"), "-o", str(OUT)], check=True)
    return OUT


_lib = None


def available() -> bool:
    return OUT.exists()


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not OUT.exists():
            raise RuntimeError(f"{OUT} not built (needs the reference sources)")
        L = C.CDLL(str(OUT))
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        L.ref_ttv.argtypes = [i, vp, vp, i, i, i]
        L.ref_normalize.argtypes = [vp, vp, i, i, i, f]
        L.ref_sensmul.argtypes = [i, vp, i, vp, vp, i, i, i, i]
        L.ref_coilsum.argtypes = [vp, vp, i, i, i, i]
        L.ref_mask.argtypes = [vp, vp, i, i, i, i]
        L.ref_abs2.argtypes = [vp, i, i, i, i]
        L.ref_abs.argtypes = [vp, vp, i, i, i]
        L.ref_rss.argtypes = [vp, vp, i, i, i, i]
        L.ref_mc.argtypes = [vp, vp, vp, vp, i, i, i, vp]
        L.ref_mc_adjoint.argtypes = [vp, vp, vp, vp, i, i, i, vp]
        _lib = L
    return _lib


def _c64(a):
    return np.ascontiguousarray(a, np.complex64)


def ttv(x: np.ndarray, forward: bool) -> np.ndarray:
    x = _c64(x)
    F, H, W = x.shape
    out = np.empty_like(x)
    lib().ref_ttv(int(forward), x.ctypes.data, out.ctypes.data, W, H, F)
    return out


def normalize(x: np.ndarray, mu: float) -> np.ndarray:
    x = _c64(x)
    F, H, W = x.shape
    out = np.empty_like(x)
    lib().ref_normalize(x.ctypes.data, out.ctypes.data, W, H, F, float(mu))
    return out


def sensmul(x: np.ndarray, S: np.ndarray, conjugate: bool, F: int | None = None) -> np.ndarray:
    x, S = _c64(x), _c64(S)
    Cc, H, W = S.shape
    Fr = x.shape[0]
    out = np.empty((Fr, Cc, H, W), np.complex64)
    lib().ref_sensmul(int(conjugate), x.ctypes.data, int(x.ndim == 4), S.ctypes.data, out.ctypes.data, W, H, Fr, Cc)
    return out


def coilsum(k: np.ndarray) -> np.ndarray:
    k = _c64(k)
    F, Cc, H, W = k.shape
    out = np.empty((F, H, W), np.complex64)
    lib().ref_coilsum(k.ctypes.data, out.ctypes.data, W, H, F, Cc)
    return out


def apply_mask(k: np.ndarray, mask: np.ndarray) -> np.ndarray:
    k = _c64(k).copy()
    m = np.ascontiguousarray(mask, np.uint8)
    F, Cc, H, W = k.shape
    lib().ref_mask(k.ctypes.data, m.ctypes.data, W, H, F, Cc)
    return k


def abs2(k: np.ndarray) -> np.ndarray:
    k = _c64(k).copy()
    F, Cc, H, W = k.shape
    lib().ref_abs2(k.ctypes.data, W, H, F, Cc)
    return k


def cabs(x: np.ndarray) -> np.ndarray:
    x = _c64(x)
    F, H, W = x.shape
    out = np.empty_like(x)
    lib().ref_abs(x.ctypes.data, out.ctypes.data, W, H, F)
    return out


def rss(k: np.ndarray) -> np.ndarray:
    k = _c64(k)
    F, Cc, H, W = k.shape
    out = np.empty((F, H, W), np.complex64)
    lib().ref_rss(k.ctypes.data, out.ctypes.data, W, H, F, Cc)
    return out


def _mc(fn, x, xn, xmesh, bb):
    x = _c64(x)
    F, H, W = x.shape
    out = np.empty_like(x)
    xn = np.ascontiguousarray(xn, np.float32)
    xm = np.ascontiguousarray(xmesh, np.int32)
    b = np.ascontiguousarray(bb, np.int32)
    fn(x.ctypes.data, out.ctypes.data, xn.ctypes.data, xm.ctypes.data, W, H, F, b.ctypes.data)
    return out


def mc(x, xn, xmesh, bb):
    """MotionCompensation with the reference's kernels (copy + interpolator)."""
    return _mc(lib().ref_mc, x, xn, xmesh, bb)


def mc_adjoint(x, xn, xmesh, bb):
    """AdjointMotionCompensation with the reference's kernels (copy, zero rectangle, adjoint interpolator)."""
    return _mc(lib().ref_mc_adjoint, x, xn, xmesh, bb)



class RegParams(C.Structure):
    """GroupwiseRegistration::InitParameters (GroupwiseRegistration.hpp:145-158)."""
    _fields_ = [("W", C.c_float), ("flagW", C.c_int), ("radius", C.c_int), ("E", C.c_int), ("Dp0", C.c_int),
                ("Dp1", C.c_int), ("nmax", C.c_int), ("et", C.c_float), ("eh", C.c_float),
                ("lambda_", C.c_float * 4)]


def registration(images: np.ndarray, radius: int = 40, E: int = 3, Dp=(4, 4), nmax: int = 100, et: float = 0.01,
                 eh: float = 0.005, lambda_=(0.0, 0.005, 0.0, 0.5), W: float = 1.0, flagW: bool = True,
                 T_init: np.ndarray | None = None) -> dict:
    """GroupwiseRegistration (init, creabspline, optimizer) on the host with the
    reference's kernels; defaults are tests/MRIRecon.cpp:121-129.  images:
    [F][N][N] complex.  Returns T [C1][C0... as the reference stores it, flat],
    xn [2][F][N][N], H [iterations + 1], bb, iterations, C0, C1, areaX, Wn."""
    x = _c64(images)
    F, N, N2 = x.shape
    assert N == N2, "square images only (the reference's mask and grid assume it)"
    L = lib()
    L.ref_registration.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(RegParams), C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    L.ref_registration.restype = C.c_int
    prm = RegParams(float(W), int(flagW), int(radius), int(E), int(Dp[0]), int(Dp[1]), int(nmax), float(et),
                    float(eh), (C.c_float * 4)(*[float(v) for v in lambda_]))
    cap = 4 * N * N * F  # more than any control grid inside the image
    T = np.zeros(cap, np.float32)
    xn = np.zeros((2, F, N, N), np.float32)
    H = np.zeros(nmax + 1, np.float32)
    bb = np.zeros(4, np.int32)
    info = np.zeros(4, np.int32)
    wn = np.zeros(1, np.float32)
    Tin = None if T_init is None else np.ascontiguousarray(T_init, np.float32).reshape(-1)
    rc = L.ref_registration(x.ctypes.data, N, F, C.byref(prm), T.ctypes.data, xn.ctypes.data, H.ctypes.data,
                            bb.ctypes.data, info.ctypes.data, wn.ctypes.data, cap,
                            None if Tin is None else Tin.ctypes.data)
    if rc != 0:
        raise ValueError("registration: unsupported geometry (grid or supports outside the image, N % 8, F < 3)")
    it, c0, c1, area = (int(v) for v in info)
    return dict(T=T[:c1 * c0 * F * 2].reshape(2, F, c0, c1), xn=xn, H=H[:it + 1], bb=bb, iterations=it, C0=c0,
                C1=c1, areaX=area, Wn=float(wn[0]))
