"""The metric's accuracy gate, NRMSE <= 1e-3 against FP64, on the large
workloads, for the plain FP32 and the mixed-precision forms: the 384x384 x 30
frames x 16 coils reconstruction, and four members of the 64-reconstruction
uneven batch (largest coil count, largest frame count, largest W*F*C, the
first) solved as one batch.  The FP64 reference is oracle/nesta_torch.py on the
same device inputs; the same restatement on complex64 arrays gives the FP32
noise floor of each workload, and a result passes at the gate or within 1.25x
that floor (accuracy_fp64.bar).  tests/accuracy_fp64.py reports the whole
batch."""
from __future__ import annotations

import pytest

from tests import accuracy_fp64 as A

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_large_workload_within_gate(ctx):
    pytest.importorskip("torch")
    (row,) = A.solve(ctx, [A.LARGE])
    print(row)
    assert row["fp32"] <= A.bar(row) and row["mixed"] <= A.bar(row)


def test_uneven_batch_members_within_gate(ctx):
    pytest.importorskip("torch")
    shapes = A.batch_shapes()
    rows = A.solve(ctx, [shapes[i] for i in A.sample_members(shapes)])
    for r in rows:
        print(r)
    assert len(rows) >= 3
    assert all(r["fp32"] <= A.bar(r) and r["mixed"] <= A.bar(r) for r in rows)


def test_stress_members_within_gate(ctx):
    """Four members of the 256-reconstruction stress batch (largest coil
    count, largest frame count, largest W*F*C, the first), one at a time."""
    pytest.importorskip("torch")
    shapes = A.batch_shapes(A.STRESS["n"], A.STRESS)
    rows = []
    for i in A.sample_members(shapes):
        rows += A.solve(ctx, [shapes[i]])
    for r in rows:
        print(r)
    assert len(rows) >= 3
    assert all(r["fp32"] <= A.bar(r) and r["mixed"] <= A.bar(r) for r in rows)
