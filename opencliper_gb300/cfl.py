"""The reference's CFL file form of KData and XData (KData.cpp:246-351,
XData.cpp:851-881), for host-side data exchange with callers of the C++
facade (include/OpenCLIPER/KData.hpp, XData.hpp).

<base>.hdr                 "W H C F" (the first line not starting with '#')
<file>                     raw complex64 k-space [F][C][H][W]
<base>_SensitivityMaps.cfl raw complex64 [C][H][W]
<base>_SamplingMasks.u32   row mask [F][H] (0/1), or
<base>_SamplingMasks.u8    pixel mask [F][H][W]
XData: <name>.cfl raw complex64 [F][H][W] and <basename(name)>.hdr "W H 1 F 1".
"""
from __future__ import annotations

import os

import numpy as np


def basename(path: str) -> str:
    """LPISupport::Utils::basename: the name without its last extension."""
    root, ext = os.path.splitext(path)
    return root if ext else path


def write_kdata(path: str, y: np.ndarray, S: np.ndarray | None = None, rowmask: np.ndarray | None = None,
                pixmask: np.ndarray | None = None) -> None:
    F, C, H, W = y.shape
    base = basename(path)
    with open(base + ".hdr", "w") as f:
        f.write(f"# W H C F\n{W} {H} {C} {F}\n")
    np.ascontiguousarray(y, np.complex64).tofile(path)
    if S is not None:
        np.ascontiguousarray(S, np.complex64).tofile(base + "_SensitivityMaps.cfl")
    if rowmask is not None:
        np.ascontiguousarray(rowmask, np.uint32).tofile(base + "_SamplingMasks.u32")
    elif pixmask is not None:
        np.ascontiguousarray(pixmask, np.uint8).tofile(base + "_SamplingMasks.u8")


def read_xdata(name: str) -> np.ndarray:
    with open(basename(name) + ".hdr") as f:
        dims = [int(v) for v in next(ln for ln in f if ln.strip() and not ln.startswith("#")).split()]
    W, H, _, F = dims[:4]
    return np.fromfile(name + ".cfl", np.complex64).reshape(F, H, W)
