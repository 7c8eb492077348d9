"""MAT-file (level 5) reader/writer of include/OpenCLIPER/gbn_matfile.hpp on
the CPU: against the two matio-written files the reference ships (its
examples/simpleMRIRecon.cpp outputs), against scipy.io-written files of every
numeric class, plain and compressed, and its DEFLATE decoder against Python's
zlib at every compression level and strategy."""
from __future__ import annotations

import os
import shutil
import subprocess
import zlib

import numpy as np
import pytest

from tests.conftest import ROOT

sio = pytest.importorskip("scipy.io")

from oracle import reference_root

REF_FILES = ["recon_fullySampled.mat", "recon_halfScan.mat"]
CLS = {6: np.float64, 7: np.float32, 8: np.int8, 9: np.uint8, 10: np.int16, 11: np.uint16, 12: np.int32,
       13: np.uint32, 14: np.int64, 15: np.uint64}


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("matfile") / "matfile_selftest"
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "matfile_selftest.cpp"), "-o", str(exe)], check=True)
    return str(exe)


def _dump(tool, path, outdir) -> dict:
    os.makedirs(outdir, exist_ok=True)
    r = subprocess.run([tool, "dump", str(path), str(outdir)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = {}
    for f in os.listdir(outdir):
        if not f.endswith(".txt"):
            continue
        name = f[:-4]
        meta = [int(t) for t in open(os.path.join(outdir, f)).read().split()]
        cls, cplx, dims = meta[0], meta[1], meta[2:]
        dt = CLS[cls]
        re = np.fromfile(os.path.join(outdir, name + ".re"), dt)
        a = re + 1j * np.fromfile(os.path.join(outdir, name + ".im"), dt) if cplx else re
        out[name] = (cls, a.reshape(dims, order="F"))
    return out


@pytest.mark.parametrize("path", REF_FILES)
def test_reads_reference_matio_files(tool, tmp_path, path):
    root = reference_root()
    if root is None or not (root / path).exists():
        pytest.skip("reference data files not available")
    path = str(root / path)
    got = _dump(tool, path, tmp_path / "d")
    want = sio.loadmat(path)
    assert set(got) == {"Dims", "XData"}
    for k in got:
        assert got[k][1].shape == want[k].shape
        assert np.array_equal(got[k][1], want[k]), k
    assert got["Dims"][0] == 13 and got["XData"][0] == 7
    # written back by the writer, read by scipy: the same variables
    r = subprocess.run([tool, "copy", path, str(tmp_path / "c.mat")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    back = sio.loadmat(str(tmp_path / "c.mat"))
    for k in ("Dims", "XData"):
        assert back[k].dtype == want[k].dtype and np.array_equal(back[k], want[k])


@pytest.mark.parametrize("compress", [False, True])
def test_reads_scipy_files_of_every_class(tool, tmp_path, compress):
    rng = np.random.default_rng(3)
    v = {
        "d": rng.standard_normal((3, 5)),
        "s": rng.standard_normal((4, 2, 3)).astype(np.float32),
        "c": (rng.standard_normal((6, 4, 2)) + 1j * rng.standard_normal((6, 4, 2))).astype(np.complex64),
        "z": rng.standard_normal((2, 3)) + 1j * rng.standard_normal((2, 3)),
        "u8": rng.integers(0, 255, (7, 3), dtype=np.uint8),
        "i16": rng.integers(-3000, 3000, (5, 5), dtype=np.int16),
        "u32": rng.integers(0, 2**32 - 1, (1, 9), dtype=np.uint32),
        "i32": rng.integers(-2**31, 2**31 - 1, (4, 1), dtype=np.int32),
        "KData_long_name": np.arange(24, dtype=np.float32).reshape(2, 3, 4),
        "txt": "not numeric",
        "cel": np.array([[np.arange(3.0)]], dtype=object),
    }
    path = tmp_path / "v.mat"
    sio.savemat(str(path), v, do_compression=compress)
    got = _dump(tool, path, tmp_path / "d")
    want = sio.loadmat(str(path))
    assert set(got) == {k for k in v if k not in ("txt", "cel")}  # character and cell variables are skipped
    for k, (cls, a) in got.items():
        assert np.array_equal(a, want[k]), k
        assert CLS[cls] == want[k].real.dtype.type, k


@pytest.mark.parametrize("level", [0, 1, 6, 9])
@pytest.mark.parametrize("strategy", [zlib.Z_DEFAULT_STRATEGY, zlib.Z_FIXED, zlib.Z_HUFFMAN_ONLY, zlib.Z_RLE])
def test_inflate_matches_zlib(tool, tmp_path, level, strategy):
    rng = np.random.default_rng(level * 10 + strategy)
    data = b"".join([
        rng.integers(0, 256, 70000, dtype=np.uint8).tobytes(),          # incompressible
        bytes(50000),                                                    # long runs
        (np.arange(40000) % 251).astype(np.uint8).tobytes(),             # periodic
        np.sin(np.arange(30000) / 50.0).astype(np.float32).tobytes(),    # float data
    ])
    c = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    z = c.compress(data) + c.flush()
    (tmp_path / "in.z").write_bytes(z)
    r = subprocess.run([tool, "inflate", str(tmp_path / "in.z"), str(tmp_path / "out.bin")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "out.bin").read_bytes() == data


def test_inflate_rejects_corruption(tool, tmp_path):
    z = bytearray(zlib.compress(b"abc" * 1000, 6))
    z[-1] ^= 0xFF  # checksum
    (tmp_path / "bad.z").write_bytes(bytes(z))
    r = subprocess.run([tool, "inflate", str(tmp_path / "bad.z"), str(tmp_path / "o")], capture_output=True, text=True)
    assert r.returncode == 1 and "checksum" in r.stderr
    (tmp_path / "not.mat").write_bytes(b"plain text, not a MAT-file" * 10)
    r = subprocess.run([tool, "dump", str(tmp_path / "not.mat"), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 1 and "MAT file" in r.stderr


def test_python_kdata_helpers_roundtrip(tmp_path):
    from opencliper_gb300 import matfile
    rng = np.random.default_rng(1)
    F, C, H, W = 3, 2, 8, 16
    y = (rng.standard_normal((F, C, H, W)) + 1j * rng.standard_normal((F, C, H, W))).astype(np.complex64)
    S = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
    matfile.write_kdata(str(tmp_path / "k.mat"), y, S, rowmask=np.ones((F, H), np.uint32))
    y2, S2 = matfile.read_kdata(str(tmp_path / "k.mat"))
    assert np.array_equal(y, y2) and np.array_equal(S, S2)
    d = sio.loadmat(str(tmp_path / "k.mat"))
    assert d["KData"].shape == (H, W, C, F) and d["SamplingMasks"].shape == (H, F)
    assert d["Dims"].ravel().tolist() == [2, 1, C, 1, F, W, H]
