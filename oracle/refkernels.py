"""The reference's own operator kernels, compiled for the host -- TEST
INFRASTRUCTURE (oracle).

build() compiles src/kernels/{hostKernelFunctions,temporalTV,
vectorNormalization,complexElementProd,xImageSum,applyMask,complexAbsPow2,
complexAbs,rss,initialize,optimizer}.cl from the reference tree, with the host shim in
oracle/refkernels/shim and the harness oracle/refkernels/harness.cpp, into
oracle/_ref/librefkernels.so.  The reference tree is only read when present
(REFERENCE_ROOT, default /root/reference); elsewhere the library is simply
unavailable and the tests that need it skip.  The functions below run the
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
REF = Path(os.environ.get("REFERENCE_ROOT", "/root/reference"))
SOURCES = ["hostKernelFunctions.cl", "temporalTV.cl", "vectorNormalization.cl", "complexElementProd.cl",
           "xImageSum.cl", "applyMask.cl", "complexAbsPow2.cl", "complexAbs.cl", "rss.cl", "initialize.cl",
           "optimizer.cl"]


def build(force: bool = False) -> Path | None:
    kdir = REF / "src" / "kernels"
    if not all((kdir / s).exists() for s in SOURCES):
        return OUT if OUT.exists() else None
    deps = [HERE / "refkernels" / "harness.cpp", HERE / "refkernels" / "shim" / "OpenCLIPER" / "kernels" /
            "hostKernelFunctions.h"] + [kdir / s for s in SOURCES]
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

