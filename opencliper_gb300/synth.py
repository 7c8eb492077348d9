"""Seeded synthetic cine MRI problems for tests and benchmarks.

No dataset is available offline, so the workloads are generated with the
shapes and value distributions of the benchmark configurations:

* phantom: 10 additive ellipses, centres uniform in the central 70 % of the
  field of view, semi-axes U(10, 80) px (scaled by min(W, H)/256 for other
  matrix sizes), rotation U(0, pi), intensities U(0.2, 1), times a smooth phase
  exp(i*phi) with phi a random 2nd-order polynomial in (u, v) in [-1, 1]^2
  rescaled to [-pi, pi];
* cine frames: each ellipse's centre and axes vary as a + 5 px *
  sin(2*pi*f/20 + phi_e) (period 20 frames, amplitude scaled like the axes);
* coils: complex Gaussian bumps (sigma = 0.4 FOV) centred on a circle of radius
  0.5 FOV at angles 2*pi*c/C with phase exp(i*2*pi*c/C), normalised so that
  sum_c |S_c|^2 = 1 per pixel;
* masks: per-frame independent Cartesian phase-encode row masks with H/R rows,
  the 16 rows around DC always sampled (rows 0..7 and H-8..H-1 in the
  unshifted layout), the rest drawn without replacement with density
  proportional to (1 - |k|/(H/2))^2, |k| = min(r, H - r);
* k-space: y = M * (FFT2_ortho(S_c x_f) + n), n complex Gaussian with
  sigma = 1e-3 * max|FFT2_ortho(S x)|, zero at unsampled positions (the forward
  model of NestaUp::operatorA with its 1/sqrt(N) scale).

Arrays follow the reference layouts: y [F][C][H][W] complex64, S [C][H][W]
complex64, pixel mask [F][H][W] uint8 (0/255), row mask [F][H] uint32.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Problem:
    y: np.ndarray        # KData [F][C][H][W] complex64
    S: np.ndarray        # SensitivityMaps [C][H][W] complex64
    mask: np.ndarray     # pixel mask [F][H][W] uint8
    rowmask: np.ndarray  # row mask [F][H] uint32
    x_true: np.ndarray   # ground-truth image series [F][H][W] complex64
    seed: int


def phantom_series(W: int, H: int, F: int, rng: np.random.Generator) -> np.ndarray:
    scale = min(W, H) / 256.0
    ne = 10
    cx = rng.uniform(0.15, 0.85, ne) * W
    cy = rng.uniform(0.15, 0.85, ne) * H
    ax = rng.uniform(10, 80, ne) * scale
    ay = rng.uniform(10, 80, ne) * scale
    rot = rng.uniform(0, np.pi, ne)
    amp = rng.uniform(0.2, 1.0, ne)
    ph = rng.uniform(0, 2 * np.pi, ne)
    # smooth phase: 2nd-order polynomial in (u, v), rescaled to [-pi, pi]
    coef = rng.standard_normal(6)
    u = np.linspace(-1, 1, W)[None, :]
    v = np.linspace(-1, 1, H)[:, None]
    phi = coef[0] + coef[1] * u + coef[2] * v + coef[3] * u * u + coef[4] * u * v + coef[5] * v * v
    phi = (phi - phi.min()) / max(phi.max() - phi.min(), 1e-12) * 2 * np.pi - np.pi
    phase = np.exp(1j * phi)
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float64)
    out = np.zeros((F, H, W), np.complex64)
    for f in range(F):
        img = np.zeros((H, W))
        wob = 5.0 * scale * np.sin(2 * np.pi * f / 20.0 + ph)
        for e in range(ne):
            c, s = np.cos(rot[e]), np.sin(rot[e])
            dx, dy = xx - (cx[e] + wob[e]), yy - (cy[e] + wob[e])
            xr, yr = c * dx + s * dy, -s * dx + c * dy
            a, b = max(ax[e] + wob[e], 1.0), max(ay[e] + wob[e], 1.0)
            img += amp[e] * (((xr / a) ** 2 + (yr / b) ** 2) <= 1.0)
        out[f] = (img * phase).astype(np.complex64)
    return out


def coil_maps(W: int, H: int, C: int) -> np.ndarray:
    """C Gaussian coil sensitivities around the field of view, normalised to
    sum |S_c|^2 = 1 at every pixel.  Far from every coil (images much longer
    than wide) the Gaussians underflow; those pixels are normalised from
    exponents shifted by their largest, which leaves the others unchanged."""
    fov = float(min(W, H))
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float64)
    expo = np.empty((C, H, W), np.float64)
    ph = np.empty(C, np.complex128)
    for c in range(C):
        ang = 2 * np.pi * c / C
        px = W / 2 + 0.5 * fov * np.cos(ang)
        py = H / 2 + 0.5 * fov * np.sin(ang)
        sig = 0.4 * fov
        expo[c] = -((xx - px) ** 2 + (yy - py) ** 2) / (2 * sig * sig)
        ph[c] = np.exp(1j * ang)
    S = np.exp(expo) * ph[:, None, None]
    nrm = np.sqrt(np.sum(np.abs(S) ** 2, axis=0, keepdims=True))
    far = nrm[0] < 1e-150
    if far.any():
        Sf = np.exp(expo[:, far] - expo[:, far].max(axis=0)) * ph[:, None]
        S[:, far] = Sf
        nrm[0][far] = np.sqrt(np.sum(np.abs(Sf) ** 2, axis=0))
    S /= nrm
    return S.astype(np.complex64)


def row_masks(H: int, F: int, R: float, rng: np.random.Generator) -> np.ndarray:
    n_lines = max(16, int(round(H / R)))
    centre = np.r_[np.arange(0, 8), np.arange(H - 8, H)]
    rest = np.setdiff1d(np.arange(H), centre)
    k = np.minimum(rest, H - rest).astype(np.float64)
    dens = (1.0 - k / (H / 2.0)) ** 2 + 1e-6
    dens /= dens.sum()
    rm = np.zeros((F, H), np.uint32)
    for f in range(F):
        rm[f, centre] = 1
        extra = n_lines - len(centre)
        if extra > 0:
            pick = rng.choice(rest, size=min(extra, len(rest)), replace=False, p=dens)
            rm[f, pick] = 1
    return rm


def make_problem(W: int, H: int, F: int, C: int, R: float, seed: int, noise: float = 1e-3) -> Problem:
    rng = np.random.default_rng(np.random.PCG64(seed))
    x = phantom_series(W, H, F, rng)
    S = coil_maps(W, H, C)
    rm = row_masks(H, F, R, rng)
    mask = np.repeat((rm.astype(np.uint8) * 255)[:, :, None], W, axis=2)
    k = np.fft.fft2(x[:, None].astype(np.complex128) * S[None], axes=(-2, -1), norm="ortho")
    sig = noise * np.abs(k).max()
    k = k + sig * (rng.standard_normal(k.shape) + 1j * rng.standard_normal(k.shape)) / np.sqrt(2)
    y = np.where(mask[:, None] != 0, k, 0).astype(np.complex64)
    return Problem(y, S, mask, rm, x, seed)


def make_fully_sampled(W: int, H: int, C: int, seed: int, noise: float = 1e-3) -> Problem:
    """Config-0 style single-frame data: y_c = FFT2(S_c x) (unnormalised) + noise."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    x = phantom_series(W, H, 1, rng)
    S = coil_maps(W, H, C)
    k = np.fft.fft2(x[:, None].astype(np.complex128) * S[None], axes=(-2, -1))
    sig = noise * np.abs(k).max()
    k = k + sig * (rng.standard_normal(k.shape) + 1j * rng.standard_normal(k.shape)) / np.sqrt(2)
    mask = np.full((1, H, W), 255, np.uint8)
    return Problem(k.astype(np.complex64), S, mask, np.ones((1, H), np.uint32), x, seed)


@dataclass
class DeviceProblem:
    y: object            # DeviceArray KData [F][C][H][W] complex64
    S: object            # DeviceArray [C][H][W] complex64
    mask: object         # DeviceArray [F][H][W] uint8
    rowmask: np.ndarray  # row mask [F][H] uint32 (host)
    seed: int


class _CudaView:
    """__cuda_array_interface__ over a DeviceArray's memory with another element
    type (complex64 as float32 pairs), for zero-copy torch views."""

    def __init__(self, d, typestr: str, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(d.ptr), False),
                                         "version": 3, "strides": None}


def host_inputs(W: int, H: int, F: int, C: int, R: float, seed: int):
    """(x [F][H][W], S [C][H][W], row mask [F][H]) of make_problem's
    distributions, drawn from `seed` (a top-level function, so that process
    pools can run it)."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    x = phantom_series(W, H, F, rng)
    S = coil_maps(W, H, C)
    rm = row_masks(H, F, R, rng)
    return x, S, rm


def host_inputs_packed(prm: tuple):
    """host_inputs((W, H, F, C, R, seed)) for Pool.imap."""
    return host_inputs(*prm)


def device_problem_from(ctx, x: np.ndarray, S: np.ndarray, rm: np.ndarray, seed: int,
                        noise: float = 1e-3) -> DeviceProblem:
    """k-space formed on the device from host inputs: the library's forward
    operator (gbn_op_encode, mask * FFT2_ortho(S_c x_f)) plus masked complex
    Gaussian noise drawn by torch from `seed`."""
    import torch

    from . import api
    F, H, W = x.shape
    C = S.shape[0]
    mask = np.repeat((rm.astype(np.uint8) * 255)[:, :, None], W, axis=2)
    dx, dS, dm = ctx.to_device(x), ctx.to_device(S), ctx.to_device(mask)
    dy = ctx.empty((F, C, H, W), np.complex64)
    api.op_encode(ctx, dx, dS, dm, dy)
    ctx.sync()
    dev = torch.device("cuda", ctx.device)
    k = torch.as_tensor(_CudaView(dy, "<f4", (F, C, H, W, 2)), device=dev)
    m = torch.as_tensor(_CudaView(dm, "|u1", (F, H, W)), device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    sig = float(noise) * float(k.square().sum(-1).sqrt().max())
    for f in range(F):  # one frame at a time bounds the temporary
        n = torch.randn(k[f].shape, generator=gen, device=dev) * (sig / np.sqrt(2.0))
        k[f] += n * (m[f] != 0)[None, :, :, None]
    torch.cuda.synchronize(dev)
    dx.free()
    return DeviceProblem(dy, dS, dm, rm, int(seed))


def make_problem_device(ctx, W: int, H: int, F: int, C: int, R: float, seed: int,
                        noise: float = 1e-3) -> DeviceProblem:
    """The distributions of make_problem with the k-space formed on the device
    (device_problem_from).  For benchmark workloads too large to generate with
    numpy FFTs; the noise stream differs from make_problem's."""
    x, S, rm = host_inputs(W, H, F, C, R, seed)
    return device_problem_from(ctx, x, S, rm, seed, noise)


def make_motion(W: int, H: int, F: int, seed: int, amplitude: float = 1.2, border: int = 4):
    """A seeded smooth stand-in for a motion estimate, in the layouts of
    ArgumentsMotionCompensation (include/OpenCLIPER/processes/
    GroupwiseRegistration.hpp:95-100): returns (xn [2][F][H][W] float32 deformed
    mesh, xmesh [2][W][H] int32 original mesh, bb [4] int32 bounding box), all
    1-based.  The original mesh is the identity; each frame's deformed mesh adds
    sinusoidal sub-pixel displacements of at most `amplitude` pixels; the
    bounding box sits `border` pixels inside the margins (H/40, W/40) that the
    interpolator adds around it, so every interpolation stays in the image."""
    rng = np.random.default_rng(seed)
    m0, m1 = H // 40, W // 40
    # rectangle rows bb1-m0-2 .. bb3+m0-1 and columns bb0-m1-2 .. bb2+m1-1 (0-based)
    bb = np.array([m1 + 2 + border, m0 + 2 + border, W - m1 - border, H - m0 - border], np.int32)
    xmesh = np.empty((2, W, H), np.int32)
    xmesh[0] = np.arange(W)[:, None] + 1  # horizontal = column + 1
    xmesh[1] = np.arange(H)[None, :] + 1  # vertical = row + 1
    rr, cc = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    xn = np.empty((2, F, H, W), np.float32)
    for f in range(F):
        ph = rng.uniform(0, 2 * np.pi, 4)
        dx = amplitude * np.sin(2 * np.pi * rr / H + ph[0]) * np.cos(2 * np.pi * cc / W + ph[1])
        dy = amplitude * np.cos(2 * np.pi * rr / H + ph[2]) * np.sin(2 * np.pi * cc / W + ph[3])
        xn[0, f] = (cc + 1 + dx).astype(np.float32)
        xn[1, f] = (rr + 1 + dy).astype(np.float32)
    return xn, xmesh, bb
