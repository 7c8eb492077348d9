"""Host-side logic without a GPU: synthetic workload properties, benchmark
helpers, and the multi-process (replica) bench path with gloo ranks."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from opencliper_gb300 import synth


def test_synthetic_problem_properties():
    p = synth.make_problem(64, 48, 5, 6, 4, seed=0)
    F, C, H, W = p.y.shape
    assert (F, C, H, W) == (5, 6, 48, 64)
    assert p.y.dtype == np.complex64 and p.S.dtype == np.complex64 and p.mask.dtype == np.uint8
    assert np.allclose(np.sum(np.abs(p.S) ** 2, axis=0), 1.0, atol=1e-5)
    for f in range(F):
        rows = np.flatnonzero(p.rowmask[f])
        assert len(rows) == max(16, round(H / 4))
        assert set(range(8)) | set(range(H - 8, H)) <= set(rows)
    assert np.all(p.y[np.broadcast_to(p.mask[:, None] == 0, p.y.shape)] == 0)
    assert np.array_equal(p.mask, np.repeat((p.rowmask * 255).astype(np.uint8)[:, :, None], W, axis=2))


@pytest.mark.parametrize("W,H,C", [(16, 512, 3), (512, 8, 4), (256, 256, 12)])
def test_coil_maps_normalised_at_every_aspect_ratio(W, H, C):
    """Pixels far from every coil (16 x 512) stay finite and normalised."""
    S = synth.coil_maps(W, H, C)
    assert S.shape == (C, H, W) and np.isfinite(S).all()
    assert np.allclose(np.sum(np.abs(S.astype(np.complex128)) ** 2, axis=0), 1.0, atol=1e-6)


def test_synthetic_problem_is_seeded():
    a = synth.make_problem(32, 32, 3, 2, 4, seed=9)
    b = synth.make_problem(32, 32, 3, 2, 4, seed=9)
    assert np.array_equal(a.y, b.y) and np.array_equal(a.mask, b.mask)


def test_algorithmic_bytes():
    import bench
    G = 640
    assert bench.algorithmic_bytes("rows", G) == 3 * 8 * G * 12 * 256 + G * 256
    assert bench.algorithmic_bytes("fwd_cols", G) == 8 * 65536 * 20 + 8 * 65536 * 12 + 8 * G * 12 * 256


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    d = bench.Dist()
    d.barrier()
    m = d.max(float(rank + 1) * 10.0)
    d.barrier()
    d.close()
    q.put((rank, m))


def test_replica_barrier_and_max_over_gloo_ranks():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert res == {0: 20.0, 1: 20.0}


_RANK_SCRIPT = '''
import json, os, sys
sys.path.insert(0, {root!r})
import bench
d = bench.Dist()
d.barrier()
t = d.max(1.0 + d.rank)
d.barrier()
if d.rank == 0:
    print(json.dumps({{"n_gpus": d.ws, "max": t, "local_ranks": d.ws}}), flush=True)
d.close()
'''


def test_gpus_flag_launches_one_rank_per_gpu(tmp_path, capfd):
    """bench.py --gpus N without a launcher starts N ranks through
    torch.distributed.run; here the ranks run a small script doing the bench's
    gloo barrier and max instead of the GPU workload."""
    pytest.importorskip("torch")
    import json

    import bench
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = tmp_path / "ranks.py"
    script.write_text(_RANK_SCRIPT.format(root=root))
    rc = bench.relaunch_ranks(2, [], script=str(script))
    assert rc == 0
    lines = [ln for ln in capfd.readouterr().out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["n_gpus"] == 2 and out["max"] == 2.0


def test_reference_arm_line(monkeypatch):
    """bench.py --impl reference: the line's contract (the reference's metric,
    unit and config, the measured steps within the wall-clock budget, the
    e2e object with no host-device copies, the cpu_baseline describing the
    run).  The whole-reconstruction timing is stubbed: one reconstruction of
    the headline workload takes ~17 s of CPU."""
    import argparse

    import bench
    calls, clock = [], [0.0]

    def fake_recon():
        calls.append(1)
        clock[0] += 0.25
        return 0.25

    monkeypatch.setattr(bench.time, "perf_counter", lambda: clock[0])
    monkeypatch.setattr(bench, "cpu_port_recon", fake_recon)
    monkeypatch.setattr(bench, "_ref_problem", lambda: None)
    monkeypatch.setattr(bench, "REF_BUDGET_S", 0.6)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    out = bench.run_reference(argparse.Namespace(steps=5), bench.Dist())
    assert out["impl"] == "reference" and out["metric"] == bench.METRIC and out["unit"] == bench.UNIT
    assert out["config"] == bench.workload_config()
    # one warm-up, then steps while the next one still fits the budget
    assert out["steps_requested"] == 5 and out["steps"] == 2 and len(calls) == 3
    assert out["value"] == 4.0 and out["ms_per_step"] == 250.0 and out["higher_is_better"] is True
    assert out["e2e"] == {"value": 4.0, "unit": bench.UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = out["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == 4.0 and cb["cores"] >= 1 and cb["sample"]
