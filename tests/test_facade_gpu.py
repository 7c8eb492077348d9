"""The OpenCLIPER-style C++ facade (include/OpenCLIPER/) driving NESTA and
SimpleMRIRecon like the reference's tests/MRIRecon.cpp, compiled with g++
against libgbnesta.so, must give the same results as the C ABI used directly."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

import opencliper_gb300 as g
from opencliper_gb300 import api, synth
from oracle import drand48
from oracle import motion as M
from tests.conftest import ROOT, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(tmp_path_factory, built_lib):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("facade") / "mrirecon_facade"
    libdir = os.path.join(ROOT, "opencliper_gb300")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-pthread", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "mrirecon_facade.cpp"), "-L", libdir, "-lgbnesta",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return exe


def test_facade_matches_c_abi(ctx, driver, tmp_path):
    W, H, F, C = 48, 40, 5, 3
    p = synth.make_problem(W, H, F, C, 4, seed=44)
    np.array([W, H, F, C], np.uint32).tofile(tmp_path / "dims.u32")
    p.y.tofile(tmp_path / "y.c64")
    p.S.tofile(tmp_path / "S.c64")
    p.rowmask.astype(np.uint32).tofile(tmp_path / "rowmask.u32")
    xn, xm, bb = synth.make_motion(W, H, F, seed=5)
    xn.astype(np.float32).tofile(tmp_path / "xn.f32")
    xm.astype(np.int32).tofile(tmp_path / "xmesh.i32")
    np.asarray(bb, np.uint32).tofile(tmp_path / "bb.u32")
    r = subprocess.run([str(driver), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    x_cpp = np.fromfile(tmp_path / "x.c64", np.complex64).reshape(F, H, W)
    simple_cpp = np.fromfile(tmp_path / "simple.c64", np.complex64).reshape(F, H, W)
    lines = (tmp_path / "stats.txt").read_text().split("\n")
    normU, iters, tolvar = lines[0].split()
    normU_mc, iters_mc, status_mc = lines[1].split()
    assert lines[2] == "refused bound_box"

    # the same through the C ABI (fresh drand48 state, like the facade program's new context)
    ctx.seed48(drand48.state_to_seed16v(drand48.DEFAULT_STATE))
    prm = g.nesta_params(lambda_i=1e-2, mu_f=3e-4, La=1.0, maxIntIter=4, maxIter=30, stoptest=1, miniter=7, tolVar=3e-4)
    x_c, st = g.nesta_run_host(ctx, p.y, p.S, p.mask, prm)
    assert np.array_equal(x_cpp, x_c)
    assert int(iters) == st["inner_iters"]
    assert abs(float(tolvar) - 3e-4) < 1e-9
    out = ctx.empty((F, H, W), np.complex64)
    api.simple_recon(ctx, ctx.to_device(p.y), ctx.to_device(p.S), out)
    assert rel_l2(simple_cpp, out.get()) == 0.0

    # motion compensation: the operators on x, then NestaUp with argsMC from x
    mc_cpp = np.fromfile(tmp_path / "mc.c64", np.complex64).reshape(F, H, W)
    mcadj_cpp = np.fromfile(tmp_path / "mcadj.c64", np.complex64).reshape(F, H, W)
    assert np.array_equal(mc_cpp, M.warp(x_cpp, xn, xm, bb))
    assert np.array_equal(mcadj_cpp, M.warp_adjoint(x_cpp, xn, xm, bb))
    dy, dS, dm = ctx.to_device(p.y), ctx.to_device(p.S), ctx.to_device(p.mask)
    prob = g.Problem(ctx, dy, dS, dm)
    prob.set_motion(ctx.to_device(xn), ctx.to_device(xm), bb)
    xmc = ctx.to_device(x_cpp)
    st_mc = prob.run(g.nesta_params(lambda_i=1e-2, mu_f=3e-4, La=1.0, maxIntIter=1, maxIter=20, stoptest=0,
                                    miniter=7, tolVar=3e-4), xmc)
    prob.close()
    xmc_cpp = np.fromfile(tmp_path / "xmc.c64", np.complex64).reshape(F, H, W)
    assert int(status_mc) == 0 and st_mc["status"] == 0
    assert int(iters_mc) == st_mc["inner_iters"]
    # deterministic: the facade's solve and the C ABI's agree bit for bit
    assert float(normU_mc) == pytest.approx(st_mc["normU"], rel=1e-5)  # printed with 6 digits
    assert np.array_equal(xmc_cpp, xmc.get())


@pytest.mark.parametrize("mask_form", ["rowmask", "pixelmask"])
def test_facade_cfl_files(ctx, tmp_path, mask_form):
    """KData(app, fileName) from the reference's CFL form (row mask file),
    SimpleMRIRecon, SimpleMRIReconSOS and NestaUp through the facade, results
    written by XData::saveCFLData and checked against the oracle."""
    from opencliper_gb300 import cfl
    from oracle import nesta_ref as R
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "cfl_facade"
    libdir = os.path.join(ROOT, "opencliper_gb300")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-pthread", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "cfl_facade.cpp"), "-L", libdir, "-lgbnesta",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    W, H, F, C = 32, 24, 4, 3
    p = synth.make_problem(W, H, F, C, 2, seed=31)
    kfile = str(tmp_path / "series.cfl")
    if mask_form == "rowmask":
        cfl.write_kdata(kfile, p.y, p.S, rowmask=p.rowmask)
    else:  # <base>_SamplingMasks.u8 with every other column of each sampled row left out
        pm = p.mask.copy()
        pm[:, :, 1::2] = 0
        p = synth.Problem(np.where(pm[:, None] != 0, p.y, 0).astype(np.complex64), p.S, pm, p.rowmask, p.x_true,
                          p.seed)
        cfl.write_kdata(kfile, p.y, p.S, pixmask=pm)
    r = subprocess.run([str(exe), kfile, str(tmp_path / "out")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    simple = cfl.read_xdata(str(tmp_path / "out_simple"))
    sos = cfl.read_xdata(str(tmp_path / "out_sos"))
    nesta = cfl.read_xdata(str(tmp_path / "out_nesta"))
    y64 = p.y.astype(np.complex128)
    assert rel_l2(simple, R.simple_recon(y64, p.S.astype(np.complex128))) < 1e-5
    assert rel_l2(sos, R.simple_recon_sos(y64)) < 1e-5
    r64 = R.nesta(p.y, p.S, p.mask, R.NestaParams(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=20,
                                                   stoptest=0, miniter=7, tolVar=3e-4), "f64")
    r32 = R.nesta(p.y, p.S, p.mask, R.NestaParams(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=20,
                                                   stoptest=0, miniter=7, tolVar=3e-4), "f32")
    assert R.nrmse(nesta, r64.x) <= 2.0 * R.nrmse(r32.x, r64.x) + 5e-6
    hdr = (tmp_path / "out_nesta.hdr").read_text().split()
    assert hdr == [str(W), str(H), "1", str(F), "1"]


@pytest.mark.parametrize("mask_form", ["rowmask", "pixelmask"])
def test_facade_mat_files(ctx, tmp_path, mask_form):
    """KData(app, "x.mat") (compressed MAT-file with Dims, KData,
    SensitivityMaps and a row-mask SamplingMasks, as KData.cpp:276-435 reads
    it), SimpleMRIRecon and NestaUp through the facade, results written by
    XData::matlabSave and KData::matlabSave and read back with scipy.io;
    XData(app, "x.mat") reloads the saved image exactly."""
    pytest.importorskip("scipy.io")
    from opencliper_gb300 import matfile
    from oracle import nesta_ref as R
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "mat_facade"
    libdir = os.path.join(ROOT, "opencliper_gb300")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-pthread", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "mat_facade.cpp"), "-L", libdir, "-lgbnesta",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    W, H, F, C = 40, 32, 4, 3
    p = synth.make_problem(W, H, F, C, 2, seed=17)
    kfile = str(tmp_path / "series.mat")
    if mask_form == "rowmask":
        matfile.write_kdata(kfile, p.y, p.S, rowmask=p.rowmask)
    else:  # uint8 pixel mask H x W x F; every other column of each sampled row left out
        pm = p.mask.copy()
        pm[:, :, 1::2] = 0
        p = synth.Problem(np.where(pm[:, None] != 0, p.y, 0).astype(np.complex64), p.S, pm, p.rowmask, p.x_true,
                          p.seed)
        matfile.write_kdata(kfile, p.y, p.S, pixelmask=pm)
    out = str(tmp_path / "out")
    r = subprocess.run([str(exe), kfile, out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "out_stats.txt").read_text().split() == ["reload", "0", "async", "invalid_argument"]
    simple = matfile.read_xdata(out + "_simple.mat")
    nesta = matfile.read_xdata(out + "_nesta.mat")
    y2, S2 = matfile.read_kdata(out + "_k.mat")
    assert np.array_equal(y2, p.y) and np.array_equal(S2, p.S.astype(np.complex64))
    import scipy.io as sio
    assert sio.loadmat(out + "_simple.mat")["Dims"].ravel().tolist() == [2, 1, 0, 1, F, W, H]
    assert rel_l2(simple, R.simple_recon(p.y.astype(np.complex128), p.S.astype(np.complex128))) < 1e-5
    prm = R.NestaParams(lambda_i=0.01, mu_f=1e-3, La=1.0, maxIntIter=1, maxIter=20, stoptest=0, miniter=7, tolVar=3e-4)
    r64 = R.nesta(p.y, p.S, p.mask, prm, "f64")
    r32 = R.nesta(p.y, p.S, p.mask, prm, "f32")
    assert R.nrmse(nesta, r64.x) <= 2.0 * R.nrmse(r32.x, r64.x) + 5e-6


def test_facade_registration_motion_loop(ctx, tmp_path, built_lib):
    """GroupwiseRegistration through the C++ facade in MRIRecon's motion-loop
    shape (tests/MRIRecon.cpp:204-282): two launches, the second started from
    the first's TData, then MotionCompensation with the estimate.  Results
    are the C ABI's bit for bit."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "registration_facade"
    libdir = os.path.join(ROOT, "opencliper_gb300")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-pthread", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "registration_facade.cpp"), "-L", libdir, "-lgbnesta",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    N, F, radius, nmax = 64, 5, 14, 4
    img = synth.phantom_series(N, N, F, np.random.default_rng(9)).astype(np.complex64)
    np.array([N, F, radius, nmax], np.uint32).tofile(tmp_path / "dims.u32")
    img.tofile(tmp_path / "x.c64")
    subprocess.run([str(exe), str(tmp_path)], check=True)
    prm = api.registration_params(W=0.05, radius=radius, nmax=nmax)
    x = ctx.to_device(img)
    r1 = api.registration(ctx, x, prm)
    r2 = api.registration(ctx, x, prm, r1["T"])
    cp = r1["cp"]
    for k, r in ((1, r1), (2, r2)):
        np.testing.assert_array_equal(np.fromfile(tmp_path / f"T{k}.f32", np.float32).reshape(2, F, cp, cp), r["T"].get())
        np.testing.assert_array_equal(np.fromfile(tmp_path / f"xn{k}.f32", np.float32).reshape(2, F, N, N), r["xn"].get())
        np.testing.assert_array_equal(np.fromfile(tmp_path / f"H{k}.f32", np.float32), r["H"])
    np.testing.assert_array_equal(np.fromfile(tmp_path / "xmesh.i32", np.int32).reshape(2, N, N), r2["xmesh"].get())
    assert np.fromfile(tmp_path / "bb.u32", np.uint32).tolist() == list(r2["bound_box"])
    mc = ctx.empty((F, N, N), np.complex64)
    api.op_motion(ctx, 1, x, mc, r2["xn"], r2["xmesh"], r2["bound_box"])  # forward (GBN_TTV_FORWARD)
    np.testing.assert_array_equal(np.fromfile(tmp_path / "mc.c64", np.complex64).reshape(F, N, N), mc.get())
    lines = (tmp_path / "stats.txt").read_text().split("\n")
    assert lines[0].split()[1] == "0" and int(lines[0].split()[2]) == cp
    assert lines[2] == "refused"
