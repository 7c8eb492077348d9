"""Host-side check of the register DFTs and the two-pass split of every
supported length (tests/cpp/fft_selftest.cu, compiled for the CPU)."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT


def test_fft_split_selftest(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / "fft_selftest"
    src = os.path.join(ROOT, "tests", "cpp", "fft_selftest.cu")
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-O2", "-x", "cu", src, "-o", str(exe)],
                   check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "ALL OK" in r.stdout
