"""The row-local kernel's per-length shape rules (rowlocal.cuh), checked on
the host: a small program built with nvcc prints, for every length the
row-local iteration takes, its factors, threads per CTA, shared-memory bytes,
CTAs per SM that shared memory allows, tensor-memory columns and staged-row
capacity.  The invariants: every layout fits a CTA's 227 KB, the tensor-memory
CTAs that shared memory lets share an SM never need more than the SM's 512
columns (so an allocation never waits on a co-resident CTA of the same
kernel), those lengths keep their state on warps 0-3 (one pass-1 item per
thread of 128), thread counts are whole warps, and the row capacity covers
every Cartesian mask at R >= 4."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    return None


def test_rowlocal_shape_rules(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = tmp_path / "rowlocal_shapes"
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "opencliper_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "rowlocal_shapes.cu"), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    rows = [tuple(int(v) for v in line.split()) for line in out.splitlines() if line.strip()]
    sizes = {r[0] for r in rows}
    # the lengths the GPU tests expect to run the row-local iteration
    from tests.test_nesta_gpu import LENGTHS, THREE_PASS_ONLY
    assert sizes == set(LENGTHS) - THREE_PASS_ONLY
    for L, A, B, nt, nbytes, ctas, tcols, rcap in rows:
        assert A * B == L
        assert nbytes <= 227 * 1024 and ctas >= 1, L
        assert nt % 32 == 0 and 32 <= nt <= 256, L
        assert rcap >= L // 4 and rcap >= min(L, 32), L
        if tcols:
            assert 8 * B == 128, L               # pass-1 / pass-3 items on warps 0-3
            assert tcols * ctas <= 512, L        # tensor memory of the co-resident CTAs
            assert nt >= 128, L
