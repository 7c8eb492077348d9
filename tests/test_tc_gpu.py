"""tcgen05 building blocks (opencliper_gb300/csrc/tc.cuh) against a
double-precision host GEMM: descriptor layouts, the kind::f16 instruction
descriptor, TMEM allocation and tcgen05.ld lane/column mapping
(tests/cpp/tc_selftest.cu, built for sm_103a)."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT

pytestmark = pytest.mark.gpu


def test_tcgen05_gemm_selftest(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "tc_selftest"
    src = os.path.join(ROOT, "tests", "cpp", "tc_selftest.cu")
    inc = os.path.join(ROOT, "opencliper_gb300", "csrc")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-I", inc, src,
                    "-o", str(exe)], check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "ALL OK" in r.stdout
