"""CFL file form (opencliper_gb300/cfl.py) as the reference lays it out:
header text, raw complex64 data, maps and mask files next to it."""
from __future__ import annotations

import numpy as np

from opencliper_gb300 import cfl


def test_kdata_files_layout(tmp_path):
    rng = np.random.default_rng(0)
    F, C, H, W = 3, 2, 8, 16
    y = (rng.standard_normal((F, C, H, W)) + 1j * rng.standard_normal((F, C, H, W))).astype(np.complex64)
    S = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
    rm = (rng.random((F, H)) > 0.5).astype(np.uint32)
    path = str(tmp_path / "k.cfl")
    cfl.write_kdata(path, y, S, rowmask=rm)
    lines = [ln for ln in (tmp_path / "k.hdr").read_text().splitlines() if not ln.startswith("#")]
    assert lines[0].split() == [str(W), str(H), str(C), str(F)]
    assert np.array_equal(np.fromfile(path, np.complex64).reshape(y.shape), y)
    assert np.array_equal(np.fromfile(tmp_path / "k_SensitivityMaps.cfl", np.complex64).reshape(S.shape), S)
    assert np.array_equal(np.fromfile(tmp_path / "k_SamplingMasks.u32", np.uint32).reshape(rm.shape), rm)
    assert cfl.basename("a/b.c/d.cfl") == "a/b.c/d" and cfl.basename("noext") == "noext"


def test_xdata_read(tmp_path):
    x = np.arange(2 * 4 * 8, dtype=np.float32).view(np.complex64).reshape(2, 4, 4)
    name = str(tmp_path / "img")
    x.tofile(name + ".cfl")
    (tmp_path / "img.hdr").write_text("4 4 1 2 1\n")
    assert np.array_equal(cfl.read_xdata(name), x)
