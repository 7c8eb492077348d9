"""MAT-file (level 5) forms of the reference's data objects, for Python
callers and tests (scipy.io does the file format):

* write_kdata(path, y, S=None, rowmask=None, pixelmask=None): the variables
  KData(app, "x.mat") reads (KData.cpp:276-435): Dims, KData, SensitivityMaps,
  SamplingMasks;
* read_xdata(path) -> [F][H][W] complex64 from XData::matlabSave's file
  (XData.cpp:886-930);
* read_kdata(path) -> (y, S or None) from KData::matlabSave's file.

Layouts: MATLAB dims are (H, W, ...) where this library's arrays are
row-major [..][H][W]; Dims = uint32 [2, 1, C, 1, F, W, H]."""
from __future__ import annotations

import numpy as np


def _sio():
    try:
        import scipy.io as sio
    except ImportError as e:  # pragma: no cover - scipy is part of the supported environment
        raise RuntimeError("MAT-file helpers need scipy") from e
    return sio


def dims(W: int, H: int, C: int, F: int) -> np.ndarray:
    return np.array([[2, 1, C, 1, F, W, H]], np.uint32)


def write_kdata(path: str, y: np.ndarray, S: np.ndarray | None = None, rowmask: np.ndarray | None = None,
                pixelmask: np.ndarray | None = None, compress: bool = True) -> None:
    """y [F][C][H][W] complex, S [C][H][W], rowmask [F][H] (nonzero = sampled
    phase-encode line) or pixelmask [F][H][W] uint8."""
    F, C, H, W = y.shape
    v = {"Dims": dims(W, H, C, F), "KData": np.ascontiguousarray(y.astype(np.complex64).transpose(2, 3, 1, 0))}
    if S is not None:
        v["SensitivityMaps"] = S.astype(np.complex64).transpose(1, 2, 0)
    if rowmask is not None:
        v["SamplingMasks"] = np.asarray(rowmask, np.uint32).reshape(F, H).T
    elif pixelmask is not None:
        v["SamplingMasks"] = np.asarray(pixelmask, np.uint8).reshape(F, H, W).transpose(1, 2, 0)
    _sio().savemat(path, v, do_compression=compress)


def _frames(a: np.ndarray) -> np.ndarray:
    a = np.asarray(a)
    if a.ndim == 2:
        a = a[:, :, None]
    return a


def read_xdata(path: str) -> np.ndarray:
    d = _sio().loadmat(path)
    x = _frames(d["XData"]).astype(np.complex64)
    return np.ascontiguousarray(x.transpose(2, 0, 1))


def read_kdata(path: str) -> tuple[np.ndarray, np.ndarray | None]:
    d = _sio().loadmat(path)
    Dm = d["Dims"].ravel()
    C, F, W, H = int(Dm[2]), int(Dm[4]), int(Dm[5]), int(Dm[6])
    k = np.asarray(d["KData"]).astype(np.complex64).reshape(H, W, max(C, 1), F, order="F")
    y = np.ascontiguousarray(k.transpose(3, 2, 0, 1))
    S = None
    if "SensitivityMaps" in d:
        s = np.asarray(d["SensitivityMaps"]).astype(np.complex64).reshape(H, W, max(C, 1), order="F")
        S = np.ascontiguousarray(s.transpose(2, 0, 1))
    return y, S
