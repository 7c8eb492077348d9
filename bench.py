#!/usr/bin/env python3
"""Benchmark: tTV-NESTA reconstructions per second on GB300.

Workload (one step = one complete reconstruction, NestaUp::launch end to end:
kept-row analysis, x0 = E^H y, maxima, power-method norm estimate, 100 NESTA
iterations): 256 x 256 image series with 20 frames and 12 coils, Cartesian
phase-encode undersampling R = 8, mu_f = 1e-3, lambda_i = 0.01, 100 fixed
iterations, plain FP32 (complex64).  Inputs are seeded synthetic data with the
workload's shapes (no dataset is available offline).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU: one process per GPU (torchrun); every rank runs independent
replicas of the workload (the path shards only across reconstructions), no
data-path collective; value = all ranks' reconstructions / max rank time.

`--impl reference` times the reference algorithm's CPU implementation on the
host cores: the reference's OpenCL library cannot be built here, so this is
the FP32 CPU restatement of NestaUp::launch (oracle port).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "tTV-NESTA recons/s at NRMSE≤1e-3 vs FP64: mixed+batched vs plain FP32, GB300"
UNIT = "recons/s"
WL = dict(W=256, H=256, F=20, C=12, R=8, seed=0)
NESTA = dict(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=100, stoptest=0, miniter=7, tolVar=3e-4)
L2_FLUSH_BYTES = 256 << 20


def workload_config(extra: dict | None = None) -> dict:
    cfg = {"workload": "tTV-NESTA cine CS, 256x256 x 20 frames, 12 coils, R=8, 100 iterations, plain FP32",
           **{k: WL[k] for k in ("W", "H", "F", "C", "R")}, "iterations": NESTA["maxIter"],
           "mu_f": NESTA["mu_f"], "lambda_i": NESTA["lambda_i"],
           "l2": "flushed between timed steps (256 MiB device write)", "parallelism": "replicas"}
    if extra:
        cfg.update(extra)
    return cfg


DATA_DESC = ("synthetic: seeded 10-ellipse cine phantom x smooth phase, Gaussian coil maps, "
             "variable-density row masks, noise 1e-3")


# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Host-side barrier and max-reduction over ranks (gloo); no GPU collective."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo", rank=self.rank, world_size=self.ws)
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi SM clock / throttle-reason samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, local_rank: int):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        idx = vis.split(",")[local_rank] if vis else str(local_rank)
        self.lines: list[str] = []
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={idx}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.t.join(timeout=2)
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
                pw.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None, "samples": len(sm), "reasons": sorted(reasons)}


def measured_peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def algorithmic_bytes(kind: str, G: int, shape: tuple | None = None) -> int:
    """Compulsory DRAM bytes of one launch of a fused kernel (complex64 = 8 B)
    on a (W, H, F, C) problem with G kept rows (default: the headline workload)."""
    W, H, F, C = shape if shape is not None else (WL["W"], WL["H"], WL["F"], WL["C"])
    N = W * H
    X, Sb, T = 8 * N * F, 8 * N * C, 8 * G * C * W
    if kind == "fwd_cols":   # x_k, S in; kept rows of DFT_H(S x) out
        return X + Sb + T
    if kind == "rows":       # T in, kept rows of y and mask in, T out
        return T + T + G * W + T
    if kind == "inv_cols":   # T, S, x_k, x_ref, w in; x_{k+1}, w out
        return T + Sb + 3 * X + 2 * X
    if kind == "iter":       # row-local iteration: IDFT_W(y) of the kept rows, S, x_k, x_ref, w_k in; x_{k+1}, w_{k+1} out
        return T + Sb + 3 * X + 2 * X
    raise KeyError(kind)


def iteration_bytes(path: str, G: int, shape: tuple) -> int:
    """Algorithmic bytes of one inner iteration of a (W, H, F, C) problem with G
    kept rows on the given path of gbn_batch_group_info."""
    if path.startswith("row_local"):
        return algorithmic_bytes("iter", G, shape)
    return sum(algorithmic_bytes(k, G, shape) for k in ("fwd_cols", "rows", "inv_cols"))


def batch_paths(b) -> list:
    """The inner-iteration path of every member of a batch."""
    ng, _ = b.groups()
    out: dict = {}
    for gi in range(ng):
        info = b.group_info(gi)
        for i in info["members"]:
            out[i] = info["path"]
    return [out[i] for i in range(len(out))]


def dense_iteration_bytes() -> int:
    """Bytes one inner iteration of the reference's algorithm moves at the headline
    workload: y, S once, x_k, x_ref, w_k read, x_{k+1}, w_{k+1} written, the pixel mask."""
    W, H, F, C = WL["W"], WL["H"], WL["F"], WL["C"]
    N = W * H
    return 8 * (N * F * C + N * C + 5 * N * F) + N * F


def ncu_traffic(kind: str, field: str = "bytes_per_launch") -> float | None:
    """Per-launch figure (DRAM bytes, or warp instructions) from the committed
    ncu summary, when present."""
    p = ROOT / "profiles" / "dram_traffic.json"
    try:
        d = json.loads(p.read_text())
        return float(d[kind][field])
    except (OSError, KeyError, ValueError):
        return None


# ---------------------------------------------------------------------------
def run_ours(args, dist: Dist) -> dict | None:
    import torch

    import opencliper_gb300 as g
    from opencliper_gb300 import synth

    torch.cuda.set_device(dist.local)
    # one explicit stream for the library, the L2 flush and the timing events
    # (the legacy default stream would not order them with the library's work)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    prob_h = synth.make_problem(WL["W"], WL["H"], WL["F"], WL["C"], WL["R"], seed=WL["seed"] + dist.rank)
    ctx = g.Context(dist.local)
    ctx.set_stream(stream.cuda_stream)
    for kv in args.tuning:
        key, val = kv.split("=", 1)
        ctx.set_tuning(key, int(val))
    y, S, m = ctx.to_device(prob_h.y), ctx.to_device(prob_h.S), ctx.to_device(prob_h.mask)
    x = ctx.empty((WL["F"], WL["H"], WL["W"]), np.complex64)
    prob = g.Problem(ctx, y, S, m)
    prm = g.nesta_params(**NESTA)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    mixed = args.precision == "mixed"
    if mixed:
        # the same reconstruction in the mixed-precision form, as a captured batch of one
        batch = g.Batch(ctx, [prob], prm, [x], precision=g.PRECISION_MIXED)
        batch.launch()
        st = batch.stats(0)
        batch.capture()
        solve = batch.launch
    else:
        st = prob.run(prm, x, stats=True)  # first run: stats (kept rows) and warm-up

        def solve():
            prob.run(prm, x, stats=False)
    for _ in range(max(0, args.warmup - 1)):
        solve()
    torch.cuda.synchronize()

    # ---- device-resident throughput -------------------------------------
    K = args.steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dist.local)
    n0 = ctx.launch_count()
    wall0 = time.perf_counter()
    for k in range(K):
        flush.fill_(k & 0xFF)
        ev[k][0].record(stream)
        solve()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    dist.barrier()
    launches = ctx.launch_count() - n0
    t_ms = sum(a.elapsed_time(b) for a, b in ev)
    t_max = dist.max(t_ms)

    # ---- end to end through the C ABI with pinned host buffers ------------
    # Every step copies its inputs from pinned host memory and reads its image
    # back.  The copies run on the context's copy stream into the other of two
    # device buffer sets (gbn_copy_upload, double buffering), so step k+1's
    # inputs travel while step k is solved; one event pair brackets all K steps.
    # The 133 MB of inputs per step exceed L2, so no flush runs in this loop.
    import ctypes as C

    from opencliper_gb300._abi import call
    hy = torch.from_numpy(prob_h.y.view(np.float32)).pin_memory()
    hS = torch.from_numpy(prob_h.S.view(np.float32)).pin_memory()
    hm = torch.from_numpy(prob_h.mask).pin_memory()
    hx = torch.empty(x.nbytes // 4, dtype=torch.float32).pin_memory()
    bi = hy.numel() * 4 + hS.numel() * 4 + hm.numel()
    bo = x.nbytes
    y2, S2, m2 = ctx.empty(y.shape, np.complex64), ctx.empty(S.shape, np.complex64), ctx.empty(m.shape, np.uint8)
    sets = [(y, S, m), (y2, S2, m2)]
    for d, h in zip(sets[1], (hy, hS, hm)):  # the second set starts with valid data (mixed: operand sizing)
        ctx.copy_upload(d, h.data_ptr(), d.nbytes)
    ctx.sync()
    prob2 = g.Problem(ctx, y2, S2, m2)
    if mixed:
        batch2 = g.Batch(ctx, [prob2], prm, [x], precision=g.PRECISION_MIXED)
        batch2.capture()
        solvers = [solve, batch2.launch]
    else:
        solvers = [solve, lambda: prob2.run(prm, x, stats=False)]

    def upload(k):
        for d, h in zip(sets[k % 2], (hy, hS, hm)):
            ctx.copy_upload(d, h.data_ptr(), d.nbytes)

    def e2e_run(n):
        ctx.copy_wait_compute()  # the first copy starts inside the timed region
        upload(0)
        for k in range(n):
            ctx.compute_wait_copy()  # step k's inputs are on the device
            ctx.copy_wait_compute()  # the next copies wait for the solve that last read their buffers
            if k + 1 < n:
                upload(k + 1)
            solvers[k % 2]()
            call("gbn_download_async", ctx.handle, C.c_void_p(hx.data_ptr()), x.ptr, x.nbytes)

    e2e_run(2)
    ctx.sync()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    e2e_run(K)
    ctx.compute_wait_copy()
    e1.record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    t2_max = dist.max(e0.elapsed_time(e1))
    if mixed:
        batch2.close()
    prob2.close()
    for a_ in (y2, S2, m2):
        a_.free()

    # ---- live per-kernel durations for the roofline ----------------------
    ctx.profile(True)
    ctx.profile_reset()
    for _ in range(2):
        flush.fill_(1)
        prob.run(prm, x, stats=False)  # the FP32 kernels: per-kernel event groups exist on this path
    prof = ctx.profile_read()
    ctx.profile(False)
    G = int(st["kept_rows"])
    fused = {k: prof[k] for k in ("fwd_cols", "rows", "inv_cols", "iter") if prof[k][0] > 0}
    dom = max(fused, key=lambda k: fused[k][1])
    n_dom, ms_dom = fused[dom]
    avg_s = ms_dom / 1e3 / max(n_dom, 1)
    alg = algorithmic_bytes(dom, G)
    peak, peak_src = measured_peak_hbm()
    achieved = alg / avg_s / 1e9
    traffic = ncu_traffic(dom)
    total_prof = sum(v[1] for v in prof.values())
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": f"{peak_src} hbm_gbs",
            # the same launch against the dense per-iteration bytes of the reference's
            # algorithm (all of y read each iteration, pixel mask): what the reference moves
            "frac_dense_bytes": round(dense_iteration_bytes() / avg_s / 1e9 / peak, 4) if dom == "iter" else None,
            "traffic": traffic, "algorithmic_bytes_per_launch": alg, "avg_launch_us": round(avg_s * 1e6, 2),
            "share_of_step": round(ms_dom / max(total_prof, 1e-9), 3),
            "groups_us_per_launch": {k: round(v[1] * 1e3 / max(v[0], 1), 2) for k, v in prof.items()}}
    # the same kernel against the instruction-issue ceiling it is bound by: warp
    # instructions per launch (ncu) over the live launch time, against 4
    # schedulers x SMs x the sampled SM clock
    inst = ncu_traffic(dom, "warp_instructions_per_launch")
    sm_mhz = (clk or {}).get("sm_mhz") or 0
    if inst and sm_mhz:
        nsm = torch.cuda.get_device_properties(dist.local).multi_processor_count
        issue_peak = 4.0 * nsm * sm_mhz * 1e6
        roof["issue"] = {"achieved_ginst_s": round(inst / avg_s / 1e9, 1), "peak_ginst_s": round(issue_peak / 1e9, 1),
                         "frac": round(inst / avg_s / issue_peak, 4),
                         "warp_instructions_per_launch": inst, "source": "profiles/dram_traffic.json (ncu)"}

    if mixed:
        batch.close()
        roof["note"] = "roofline of the FP32 kernels; the mixed form's tensor-core kernels are profiled under profiles/"
    prob.close()
    for a in (y, S, m, x):
        a.free()
    forms = {}
    if not args.no_forms and dist.ws == 1:
        wanted = {f.strip() for f in args.forms.split(",") if f.strip()}
        for name, fn in FORMS:
            if name in wanted:
                forms[name] = fn(ctx, stream, args)
    ctx.set_stream(None)
    ctx.close()
    n = dist.ws
    out = {"metric": METRIC, "value": round(n * K / (t_max / 1e3), 3), "unit": UNIT, "n_gpus": n, "steps": K,
           "warmup": args.warmup, "ms_per_step": round(t_max / K, 4), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None,
           "dtype": "c64 (column transforms on tcgen05: split fp16 operands, fp32 accumulation)" if mixed else "c64",
           "data": DATA_DESC,
           "config": workload_config(),
           "solver": {"kept_rows": G, "precision": args.precision},
           "e2e": {"value": round(n * K / (t2_max / 1e3), 3), "unit": UNIT, "h2d_bytes_per_step": int(bi),
                   "d2h_bytes_per_step": int(bo),
                   "pipeline": "inputs of step k+1 copied on the copy stream while step k is solved"},
           "gpu_launches": int(launches), "roofline": roof, "clocks": clk,
           "wall_s_timed_region": round(wall, 3)}
    if forms:
        out["forms"] = forms
    return out


def _graph_rate(ctx, stream, batch, n: int, reps: int) -> tuple[float, float]:
    """(recons/s, ms per replay) of a captured batch, events on the library's stream."""
    import torch
    batch.capture()
    batch.launch()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for k in range(reps):
        ev[k][0].record(stream)
        batch.launch()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(c) for a, c in ev) / reps
    return n / (ms / 1e3), ms


def _nrmse(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def mixed_forms(ctx, stream, args=None, reps: int = 5) -> dict:
    """The mixed-precision form (column transforms on the tensor cores, split
    fp16 operands, FP32 accumulation) against the plain FP32 path on the
    headline workload and on the 384x384 x 30 frames x 16 coils workload, same
    inputs and drand48 state for both; NRMSE of the mixed image against the
    plain FP32 one."""
    import opencliper_gb300 as g
    from opencliper_gb300 import synth
    out = {}
    for tag, (W, H, F, Cc, Rr) in (("256x256x20c12", (256, 256, 20, 12, 8)), ("384x384x30c16", (384, 384, 30, 16, 8))):
        p = synth.make_problem_device(ctx, W, H, F, Cc, Rr, seed=7)
        prob = g.Problem(ctx, p.y, p.S, p.mask)
        x = ctx.empty((F, H, W), np.complex64)
        res, imgs = {}, {}
        for name, prec in (("fp32", g.PRECISION_FP32), ("mixed", g.PRECISION_MIXED)):
            ctx.seed48((0x330E, 0xABCD, 0x1234))
            b = g.Batch(ctx, [prob], g.nesta_params(**NESTA), [x], precision=prec)
            b.launch()
            imgs[name] = x.get()
            status = b.stats(0)["status"]
            tc_groups = b.groups()[1]
            rate, ms = _graph_rate(ctx, stream, b, 1, reps)
            res[name] = {"value": round(rate, 3), "ms_per_recon": round(ms, 3), "status": int(status),
                         "tensor_core_forward": bool(tc_groups)}
            b.close()
        res["speedup_mixed_over_fp32"] = round(res["mixed"]["value"] / res["fp32"]["value"], 3)
        res["nrmse_mixed_vs_fp32"] = float(f"{_nrmse(imgs['mixed'], imgs['fp32']):.3e}")
        res["unit"] = UNIT
        out[tag] = res
        prob.close()
        for a in (p.y, p.S, p.mask, x):
            a.free()
    return out


def motion_form(ctx, stream, args=None) -> dict:
    """The motion-compensated form (NestaUp with argsMC) on the headline
    workload: a seeded smooth motion estimate (synth.make_motion, up to 1.2 px
    displacements over the whole field of view), started from the plain
    reconstruction's image as the reference's motion-compensated pass is;
    same NESTA settings; events on the library's stream around each run, the
    starting image re-uploaded outside them.  The plain FP32 solve of the same
    problem is timed alongside."""
    import opencliper_gb300 as g
    from opencliper_gb300 import synth
    reps = args.form_reps if args is not None else 3
    W, H, F, Cc, Rr = WL["W"], WL["H"], WL["F"], WL["C"], WL["R"]
    p = synth.make_problem_device(ctx, W, H, F, Cc, Rr, seed=11)
    prob = g.Problem(ctx, p.y, p.S, p.mask)
    x = ctx.empty((F, H, W), np.complex64)
    prm = g.nesta_params(**NESTA)
    prob.run(prm, x)
    x0 = x.get()
    xn, xm, bb = synth.make_motion(W, H, F, seed=3)
    dxn, dxm = ctx.to_device(xn), ctx.to_device(xm)
    res = {"workload": f"{W}x{H} x {F} frames, {Cc} coils, R={Rr}, {NESTA['maxIter']} iterations, "
                       "motion estimate: identity mesh + sinusoidal displacements <= 1.2 px", "unit": UNIT}
    for name, mc in (("plain", False), ("motion", True)):
        prob.set_motion(dxn, dxm, bb) if mc else prob.set_motion(None, None, None)
        times, st = [], None
        for k in range(reps + 1):
            x.set(x0)
            a, c = torch_events()
            a.record(stream)
            st = prob.run(prm, x, stats=False) if k < reps else prob.run(prm, x, stats=True)
            c.record(stream)
            stream.synchronize()
            if k > 0 or reps == 0:
                times.append(a.elapsed_time(c))
        ms = sum(times) / len(times)
        res[name] = {"value": round(1e3 / ms, 3), "ms_per_recon": round(ms, 3), "status": int(st["status"]),
                     "normU": round(float(st["normU"]), 5), "normest_iters": int(st["normest_iters"])}
    res["motion_over_plain_time"] = round(res["plain"]["value"] / res["motion"]["value"], 3)
    prob.close()
    for a in (p.y, p.S, p.mask, x, dxn, dxm):
        a.free()
    return res


def registration_form(ctx, stream, args=None) -> dict:
    """GroupwiseRegistration (the motion estimation of MRIRecon's motion loop,
    MRIRecon.cpp:246-282) on the plain reconstruction of the headline problem,
    with the reference's defaults (tests/MRIRecon.cpp:121-129: radius-40 region
    of interest, cubic splines every 4 px, up to 100 iterations); then one
    motion-compensated solve with the estimated mesh.  Events on the library's
    stream around each registration.  cpu_port: oracle/registration.py (numpy,
    one core) on the same frames for two iterations, per iteration."""
    import time

    import opencliper_gb300 as g
    from opencliper_gb300 import synth
    reps = args.form_reps if args is not None else 3
    W, H, F, Cc, Rr = WL["W"], WL["H"], WL["F"], WL["C"], WL["R"]
    p = synth.make_problem_device(ctx, W, H, F, Cc, Rr, seed=11)
    prob = g.Problem(ctx, p.y, p.S, p.mask)
    x = ctx.empty((F, H, W), np.complex64)
    prm = g.nesta_params(**NESTA)
    prob.run(prm, x)
    x0 = x.get()
    rp = g.registration_params()
    times, r = [], None
    for k in range(reps + 1):
        if r is not None:
            for key in ("T", "xn", "xmesh"):
                r[key].free()
        a, c = torch_events()
        a.record(stream)
        r = g.registration(ctx, x, rp)
        c.record(stream)
        stream.synchronize()
        if k > 0 or reps == 0:
            times.append(a.elapsed_time(c))
    ms = sum(times) / len(times)
    res = {"workload": f"{W}x{H} x {F} frames (the plain reconstruction of the headline problem), radius-40 "
                       "region of interest, cubic B-splines every 4 px, nmax 100, lambda {0, 0.005, 0, 0.5}",
           "unit": "registrations/s",
           "gpu": {"value": round(1e3 / ms, 3), "ms_per_registration": round(ms, 3),
                   "iterations": int(r["iterations"]), "ms_per_iteration": round(ms / max(1, r["iterations"]), 4),
                   "kernel_launches_per_iteration": 4, "control_points": int(r["cp"]) ** 2,
                   "H0": float(r["H0"]), "H": float(r["H_final"]), "status": int(r["status"])}}
    # the motion-compensated solve with the estimated mesh
    prob.set_motion(r["xn"], r["xmesh"], r["bound_box"])
    x.set(x0)
    a, c = torch_events()
    a.record(stream)
    st = prob.run(prm, x, stats=True)
    c.record(stream)
    stream.synchronize()
    mc_ms = a.elapsed_time(c)
    res["motion_iteration"] = {"registration_plus_mc_solve_ms": round(ms + mc_ms, 3), "mc_solve_ms": round(mc_ms, 3),
                               "status": int(st["status"])}
    if args is None or not getattr(args, "no_cpu_baseline", False):
        from oracle import registration as RG
        t0 = time.perf_counter()
        cpu = RG.Registration(W, F, nmax=2).run(x0)
        dt = time.perf_counter() - t0
        per_it = dt / max(1, cpu["iterations"])
        res["cpu_port"] = {"kind": "port", "cores": 1, "sample": f"{cpu['iterations']} iterations, same frames",
                           "s_per_iteration": round(per_it, 3),
                           "projected_s_per_registration": round(per_it * max(1, r["iterations"]), 2)}
        res["speedup_per_iteration_vs_cpu_port"] = round(per_it * 1e3 / (ms / max(1, r["iterations"])), 1)
    prob.close()
    for arr in (p.y, p.S, p.mask, x, r["T"], r["xn"], r["xmesh"]):
        arr.free()
    return res


def run_forms_only(args, dist: Dist) -> dict | None:
    """The forms named by --forms on their own, without the headline timing."""
    import torch

    import opencliper_gb300 as g
    torch.cuda.set_device(dist.local)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = g.Context(dist.local)
    ctx.set_stream(stream.cuda_stream)
    for kv in args.tuning:
        key, val = kv.split("=", 1)
        ctx.set_tuning(key, int(val))
    wanted = {f.strip() for f in args.forms.split(",") if f.strip()}
    forms = {name: fn(ctx, stream, args) for name, fn in FORMS if name in wanted}
    ctx.set_stream(None)
    ctx.close()
    return {"metric": METRIC, "unit": UNIT, "forms_only": True, "forms": forms}


def torch_events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


BATCH_WL = dict(n=64, sizes=(128, 192, 256, 320, 384), frames=(12, 40), coils=(8, 32), accel=(4, 12), seed0=1000)


def batched_form(ctx, stream, args=None, reps: int = 2) -> dict:
    """The batched form on the uneven workload: 64 reconstructions, each with
    its own seed 1000+i drawing W=H from {128..384}, F ~ U{12..40},
    C ~ U{8..32}, R ~ U{4..12}, solved by one captured CUDA graph (gbn_batch_*)
    with the same NESTA settings as the headline workload, in plain FP32 and in
    the mixed form.  Device-resident inputs; events on the library's stream
    around each graph replay."""
    import opencliper_gb300 as g
    from opencliper_gb300 import synth
    B = BATCH_WL
    probs, outs, arrays, shapes = [], [], [], []
    n_units = 0
    for i in range(B["n"]):
        r = np.random.default_rng(B["seed0"] + i)
        Wd = int(r.choice(B["sizes"]))
        F = int(r.integers(B["frames"][0], B["frames"][1] + 1))
        Cc = int(r.integers(B["coils"][0], B["coils"][1] + 1))
        Rr = int(r.integers(B["accel"][0], B["accel"][1] + 1))
        p = synth.make_problem_device(ctx, Wd, Wd, F, Cc, Rr, seed=B["seed0"] + i)
        x = ctx.empty((F, Wd, Wd), np.complex64)
        probs.append(g.Problem(ctx, p.y, p.S, p.mask))
        outs.append(x)
        arrays += [p.y, p.S, p.mask, x]
        shapes.append((Wd, F, Cc, Rr))
        n_units += Wd * Wd * F * Cc
    res = {"workload": f"{B['n']} uneven reconstructions, W=H in {list(B['sizes'])}, F U{{12..40}}, "
                       f"C U{{8..32}}, R U{{4..12}}, seeds {B['seed0']}+i, one CUDA graph",
           "unit": UNIT, "pixel_coil_frames": int(n_units), "sizes_seen": sorted(set(s[0] for s in shapes))}
    # autotune one representative shape per matrix size (median frames and coils of
    # its members): launch shapes and the mixed form's forward choice per group
    reps_shape = []
    for Wd in sorted(set(s[0] for s in shapes)):
        mem = [s for s in shapes if s[0] == Wd]
        reps_shape.append((Wd, Wd, int(np.median([m[1] for m in mem])), int(np.median([m[2] for m in mem]))))
    t0 = time.perf_counter()
    ctx.autotune(reps_shape)
    res["autotune"] = {"shapes": [list(r) for r in reps_shape], "seconds": round(time.perf_counter() - t0, 1),
                       "k1_k2": [list(ctx.tuning_for(*r)) for r in reps_shape]}
    for name, prec in (("fp32", g.PRECISION_FP32), ("mixed", g.PRECISION_MIXED)):
        try:
            b = g.Batch(ctx, probs, g.nesta_params(**NESTA), outs, precision=prec)
        except g.GbnError as e:  # e.g. a frame with more kept rows than the mixed operand takes
            res[name] = {"unavailable": str(e)}
            continue
        n0 = ctx.launch_count()
        ng, ntc = b.groups()
        rate, ms = _graph_rate(ctx, stream, b, B["n"], reps)
        paths = batch_paths(b)
        res[name] = {"value": round(rate, 3), "ms_per_batch": round(ms, 2), "reps": reps,
                     "groups": ng, "tensor_core_forward_groups": ntc,
                     "members_by_path": {k: paths.count(k) for k in sorted(set(paths))},
                     "kept_rows_total": int(sum(b.stats(i)["kept_rows"] for i in range(B["n"]))),
                     "status_nonzero": int(sum(b.stats(i)["status"] != 0 for i in range(B["n"]))),
                     "host_launch_calls_per_replay": int((ctx.launch_count() - n0) // (reps + 1))}
        b.close()
    for pr in probs:
        pr.close()
    for a in arrays:
        a.free()
    return res


def cpu_port_sample(iters: int = 3) -> dict:
    """FP32 CPU restatement timed on a bounded sample: setup plus `iters` inner
    iterations of one reconstruction, extrapolated to the full 100."""
    from opencliper_gb300 import synth
    from oracle import nesta_ref as R
    p = synth.make_problem(WL["W"], WL["H"], WL["F"], WL["C"], WL["R"], seed=WL["seed"])
    prm = R.NestaParams(**{**NESTA, "maxIter": iters})
    tm: dict = {}
    t0 = time.perf_counter()
    R.nesta(p.y, p.S, p.mask, prm, "f32", timings=tm)
    wall = time.perf_counter() - t0
    per_iter = float(np.mean(tm["iters"]))
    est = tm["setup"] + NESTA["maxIter"] * per_iter
    return {"value": round(1.0 / est, 6), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": f"FP32 numpy/scipy restatement (scipy.fft workers={os.cpu_count()}): setup "
                      f"{tm['setup']:.2f} s + {iters} inner iterations ({per_iter:.3f} s each) of one "
                      f"reconstruction of this workload, extrapolated to {NESTA['maxIter']} iterations",
            "est_seconds_per_recon": round(est, 3), "sample_wall_s": round(wall, 2)}


STRESS_WL = dict(n=256, sizes=(128, 192, 256, 320, 384, 448), frames=(12, 40), coils=(8, 48), accel=(4, 12),
                 seed0=5000, device_budget_gb=230)


def stress_form(ctx, stream, args=None) -> dict:
    """The stress batch: 256 reconstructions drawn like the uneven workload but
    with W=H up to 448 and up to 48 coils (seeds 5000+i), all resident in HBM
    at once, solved by one captured CUDA graph per precision (one timed replay
    each after the capturing run).  Host inputs come from a spawn process pool;
    k-space is formed on the device.  Reports recons/s, the HBM footprint, the
    algorithmic HBM traffic rate of the fused kernels and the distribution of
    the mixed form's NRMSE against the plain FP32 images (max, p99).  If the
    drawn set would exceed device_budget_gb it is cut at that point and the cut
    is reported."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    import torch

    import opencliper_gb300 as g
    from opencliper_gb300 import synth
    B = STRESS_WL
    params = []
    for i in range(B["n"]):
        r = np.random.default_rng(B["seed0"] + i)
        Wd = int(r.choice(B["sizes"]))
        F = int(r.integers(B["frames"][0], B["frames"][1] + 1))
        Cc = int(r.integers(B["coils"][0], B["coils"][1] + 1))
        Rr = int(r.integers(B["accel"][0], B["accel"][1] + 1))
        params.append((Wd, Wd, F, Cc, Rr, B["seed0"] + i))
    # k-space, maps, masks, output and solver state per instance (bytes, approximate)
    need = [8 * W * H * F * C + 8 * W * H * C + W * H * F + 8 * W * H * F * 8 + 8 * (H // R + 16) * F * C * W
            for (W, H, F, C, R, _) in params]  # the row buffer is fitted to the kept rows (gbn_problem_fit_rows)
    keep, tot = 0, 0
    for b in need:
        if (tot + b) / 1e9 > B["device_budget_gb"]:
            break
        tot += b
        keep += 1
    params = params[:keep]
    free0, total = torch.cuda.mem_get_info()
    t0 = time.perf_counter()
    probs, outs, arrays, shapes = [], [], [], []
    oom = ""
    # spawn (the parent already holds a CUDA context); a worker that dies raises here instead of hanging
    with ProcessPoolExecutor(min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as pool:
        for (W, H, F, Cc, Rr, seed), (x, S, rm) in zip(params, pool.map(synth.host_inputs_packed, params)):
            if oom:
                continue
            try:
                p = synth.device_problem_from(ctx, x, S, rm, seed)
                arrays += [p.y, p.S, p.mask]
                xo = ctx.empty((F, H, W), np.complex64)
                arrays.append(xo)
                probs.append(g.Problem(ctx, p.y, p.S, p.mask))
                probs[-1].fit_rows(0)  # row buffer sized to the kept rows instead of the whole k-space
            except (g.GbnError, torch.cuda.OutOfMemoryError) as e:  # device full: keep what fits
                oom = str(e)
                continue
            outs.append(xo)
            shapes.append((W, H, F, Cc))
    gen_s = time.perf_counter() - t0
    if oom:
        params = params[:len(probs)]
    res = {"workload": f"{len(params)} of {B['n']} reconstructions, W=H in {list(B['sizes'])}, F U{{12..40}}, "
                       f"C U{{8..48}}, R U{{4..12}}, seeds {B['seed0']}+i, one CUDA graph per precision",
           "unit": UNIT, "instances": len(params), "generation_s": round(gen_s, 1),
           "pixel_coil_frames": int(sum(W * H * F * C for (W, H, F, C) in shapes))}
    if oom:
        res["device_full"] = oom
    ref = []
    for name, prec in (("fp32", g.PRECISION_FP32), ("mixed", g.PRECISION_MIXED)):
        ctx.seed48((0x330E, 0xABCD, 0x1234))  # both precisions replay the same drand48 sequence
        try:
            b = g.Batch(ctx, probs, g.nesta_params(**NESTA), outs, precision=prec)
        except g.GbnError as e:
            res[name] = {"unavailable": str(e)}
            continue
        free1, _ = torch.cuda.mem_get_info()
        rate, ms = _graph_rate(ctx, stream, b, len(probs), 1)
        paths = batch_paths(b)
        G = [int(b.stats(i)["kept_rows"]) for i in range(len(probs))]
        alg = sum(iteration_bytes(paths[i], Gi, sh) for i, (Gi, sh) in enumerate(zip(G, shapes))) * NESTA["maxIter"]
        res[name] = {"value": round(rate, 3), "ms_per_batch": round(ms, 1),
                     "hbm_used_gb": round((total - free1) / 1e9, 1),
                     "algorithmic_gbs": round(alg / (ms / 1e3) / 1e9, 1),
                     "members_by_path": {k: paths.count(k) for k in sorted(set(paths))},
                     "status_nonzero": int(sum(b.stats(i)["status"] != 0 for i in range(len(probs))))}
        dev = torch.device("cuda", ctx.device)
        imgs = [torch.as_tensor(synth._CudaView(o, "<f4", o.shape + (2,)), device=dev) for o in outs]
        if name == "fp32":
            ref = [t.clone() for t in imgs]
        else:
            e = torch.stack([(a - r).norm() / r.norm().clamp_min(1e-30) for a, r in zip(imgs, ref)]).cpu().numpy()
            res["nrmse_mixed_vs_fp32"] = {"max": float(f"{e.max():.3e}"), "p99": float(f"{np.percentile(e, 99):.3e}"),
                                          "median": float(f"{np.median(e):.3e}")}
        b.close()
    del ref
    for pr in probs:
        pr.close()
    for a in arrays:
        a.free()
    res["hbm_free_before_gb"] = round(free0 / 1e9, 1)
    return res


def simple_form(ctx, stream, args=None, reps: int = 50) -> dict:
    """SimpleMRIRecon (SimpleMRIRecon.cpp:80-101, the fully sampled 256x256
    single-slice reconstruction with 8 coils): x = sum_c conj(S_c) ifft2(y_c)
    through gbn_simple_recon on device-resident inputs, events on the library's
    stream around each call with a 256 MiB L2 flush between calls; algorithmic
    bytes = y + S read, x written; the FP32 CPU restatement
    (oracle.nesta_ref.simple_recon, scipy.fft on all host cores) timed beside it."""
    import torch

    from opencliper_gb300 import api, synth
    W, H, Cc = 256, 256, 8
    p = synth.make_fully_sampled(W, H, Cc, seed=0)
    dy, dS = ctx.to_device(p.y), ctx.to_device(p.S)
    x = ctx.empty((1, H, W), np.complex64)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=torch.device("cuda", ctx.device))
    for _ in range(3):
        api.simple_recon(ctx, dy, dS, x)
    stream.synchronize()
    n0 = ctx.launch_count()
    times = []
    for k in range(reps):
        flush.fill_(k & 0xFF)
        a, c = torch_events()
        a.record(stream)
        api.simple_recon(ctx, dy, dS, x)
        c.record(stream)
        times.append((a, c))
    stream.synchronize()
    launches = (ctx.launch_count() - n0) // reps
    ms = float(np.median([a.elapsed_time(c) for a, c in times]))
    alg = p.y.nbytes + p.S.nbytes + x.nbytes
    peak, peak_src = measured_peak_hbm()
    res = {"workload": f"SimpleMRIRecon, {W}x{H}, 1 frame, {Cc} coils, fully sampled, FP32", "unit": UNIT,
           "value": round(1e3 / ms, 1), "ms_per_recon": round(ms, 4), "launches_per_recon": int(launches),
           "roofline": {"bound": "hbm", "achieved": round(alg / (ms / 1e3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(alg / (ms / 1e3) / 1e9 / peak, 4), "peak_source": f"{peak_src} hbm_gbs",
                        "algorithmic_bytes": int(alg)}}
    if args is None or not getattr(args, "no_cpu_baseline", False):
        from oracle import nesta_ref as R
        R.simple_recon(p.y, p.S)
        t0 = time.perf_counter()
        n = 0
        while time.perf_counter() - t0 < 3.0:
            R.simple_recon(p.y, p.S)
            n += 1
        cpu_s = (time.perf_counter() - t0) / n
        res["cpu_baseline"] = {"value": round(1.0 / cpu_s, 2), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                               "sample": f"{n} reconstructions by the FP32 restatement (scipy.fft workers="
                                         f"{os.cpu_count()})"}
    for a_ in (dy, dS, x):
        a_.free()
    return res


# the batched form autotunes its shapes into the context: forms that should see the defaults run first
FORMS = (("simple", simple_form), ("mixed", mixed_forms), ("motion", motion_form), ("registration", registration_form),
         ("batched", batched_form), ("stress", stress_form))


REF_BUDGET_S = 300.0  # wall-clock budget of the reference arm's measured steps


def cpu_port_recon() -> float:
    """Seconds of one whole reconstruction of the headline workload by the FP32
    CPU restatement of NestaUp::launch (setup and all 100 inner iterations)."""
    from oracle import nesta_ref as R
    p = _ref_problem()
    t0 = time.perf_counter()
    R.nesta(p.y, p.S, p.mask, R.NestaParams(**NESTA), "f32")
    return time.perf_counter() - t0


_REF_P = None


def _ref_problem():
    global _REF_P
    if _REF_P is None:
        from opencliper_gb300 import synth
        _REF_P = synth.make_problem(WL["W"], WL["H"], WL["F"], WL["C"], WL["R"], seed=WL["seed"])
    return _REF_P


def run_reference(args, dist: Dist) -> dict | None:
    """The reference arm: whole reconstructions (setup + 100 iterations) by the
    FP32 restatement on the host cores, one per step.  One warm-up
    reconstruction; then up to --steps measured ones while they fit the
    REF_BUDGET_S wall-clock budget (each takes ~17 s on 16 cores), and the line
    reports how many ran."""
    if dist.rank != 0:
        return None
    _ref_problem()
    cpu_port_recon()  # warm-up: FFT plans, page-in
    times = []
    t_start = time.perf_counter()
    for _ in range(args.steps):
        times.append(cpu_port_recon())
        elapsed = time.perf_counter() - t_start
        if elapsed + times[-1] > REF_BUDGET_S:
            break
    est = float(np.mean(times))
    v = round(1.0 / est, 6)
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": dist.ws,
            "steps": len(times), "steps_requested": args.steps, "warmup": 1, "ms_per_step": round(est * 1e3, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": DATA_DESC,
            "config": workload_config(),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": f"per step one whole reconstruction (setup + {NESTA['maxIter']} inner "
                                       f"iterations) by the FP32 numpy/scipy restatement of NestaUp::launch "
                                       f"(scipy.fft workers={os.cpu_count()}); {len(times)} measured steps within a "
                                       f"{REF_BUDGET_S:.0f} s budget after one warm-up (the reference's OpenCL "
                                       "build is unavailable: no OpenCL ICD, clFFT, CLBlast)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def relaunch_ranks(n: int, argv: list[str], script: str | None = None) -> int:
    """`--gpus N` without a launcher: start N ranks of `script` (this file by
    default) with torch.distributed.run on 127.0.0.1 (one process per GPU,
    LOCAL_RANK = GPU index); rank 0 prints the JSON line."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), script or str(Path(__file__).resolve()), *argv]
    return subprocess.call(cmd)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU restatement timing")
    ap.add_argument("--no-forms", action="store_true", help="skip the mixed, batched and motion form measurements")
    ap.add_argument("--forms", default="simple,mixed,batched,motion,registration",
                    help="comma-separated forms to measure after the headline (simple, mixed, batched, motion, "
                         "registration; stress, the 256-reconstruction ~150 GB batch, only when named)")
    ap.add_argument("--forms-only", action="store_true",
                    help="measure only the forms named by --forms (no headline line; for profiling)")
    ap.add_argument("--form-reps", type=int, default=3, help="timed repetitions of the motion form")
    ap.add_argument("--precision", choices=["fp32", "mixed"], default="fp32",
                    help="form timed as the main workload (the headline is fp32)")
    ap.add_argument("--tuning", action="append", default=[], metavar="KEY=VALUE",
                    help="gbn_ctx_set_tuning knob for the main workload (repeatable)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return relaunch_ranks(args.gpus, list(sys.argv[1:] if argv is None else argv))
    dist = Dist()
    if "WORLD_SIZE" in os.environ and dist.ws != args.gpus:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={dist.ws}; reporting the {dist.ws} ranks that run",
              file=sys.stderr)
    try:
        if args.impl == "reference":
            out = run_reference(args, dist)
        elif args.forms_only:
            out = run_forms_only(args, dist)
        else:
            out = run_ours(args, dist)
            if out is not None and dist.rank == 0 and dist.ws == 1:
                out["cpu_baseline"] = (cpu_port_sample() if not args.no_cpu_baseline else
                                       {"value": None, "unit": UNIT, "cores": 0, "kind": "port",
                                        "sample": "skipped (--no-cpu-baseline)"})
    finally:
        dist.close()
    if out is not None and dist.rank == 0:
        print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
