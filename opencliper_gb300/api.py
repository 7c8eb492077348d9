"""Device context and device arrays over the C ABI (numpy on the host side)."""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _abi
from ._abi import NestaParams, NestaStats, call


class DeviceArray:
    """A device allocation owned by a Context, with a numpy-like shape/dtype."""

    def __init__(self, ctx: "Context", shape, dtype, ptr: int | None = None):
        self.ctx = ctx
        self.shape = tuple(int(s) for s in shape)
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape, dtype=np.int64)) * self.dtype.itemsize
        if ptr is None:
            p = C.c_void_p()
            call("gbn_alloc", ctx.handle, self.nbytes, C.byref(p))
            ptr = p.value
            self._owned = True
        else:
            self._owned = False
        self.ptr = int(ptr)
        ctx._children.add(self)

    @property
    def size(self) -> int:
        return int(np.prod(self.shape, dtype=np.int64))

    def get(self) -> np.ndarray:
        out = np.empty(self.shape, self.dtype)
        call("gbn_download", self.ctx.handle, out.ctypes.data, self.ptr, self.nbytes)
        return out

    def set(self, arr: np.ndarray) -> "DeviceArray":
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        if a.nbytes != self.nbytes:
            raise ValueError(f"size mismatch: {a.nbytes} bytes into {self.nbytes}")
        call("gbn_upload", self.ctx.handle, self.ptr, a.ctypes.data, self.nbytes)
        self.ctx.sync()  # the host array may go away after return
        return self

    def zero(self) -> "DeviceArray":
        call("gbn_memset", self.ctx.handle, self.ptr, 0, self.nbytes)
        return self

    def free(self) -> None:
        if self._owned and self.ptr and self.ctx.handle:
            call("gbn_free", self.ctx.handle, self.ptr)
        self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """One device and one stream (the reference's CLapp, src/CLapp.cpp:188-575)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        call("gbn_ctx_create", int(device), C.byref(h))
        self.handle = h.value
        self.device = device
        self._children = weakref.WeakSet()  # batches, problems and arrays of this context

    def close(self) -> None:
        if self.handle:
            # objects that refer to the context go first, whatever order the
            # garbage collector would pick
            kids = list(self._children)
            for kind in (Batch, Problem, DeviceArray):
                for k in kids:
                    if isinstance(k, kind):
                        k.close() if kind is not DeviceArray else k.free()
            call("gbn_ctx_destroy", self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # memory -----------------------------------------------------------
    def empty(self, shape, dtype) -> DeviceArray:
        return DeviceArray(self, shape, dtype)

    def zeros(self, shape, dtype) -> DeviceArray:
        return DeviceArray(self, shape, dtype).zero()

    def to_device(self, arr: np.ndarray) -> DeviceArray:
        a = np.ascontiguousarray(arr)
        d = DeviceArray(self, a.shape, a.dtype)
        return d.set(a)

    def sync(self) -> None:
        call("gbn_ctx_sync", self.handle)

    # prefetch on the context's copy stream (gbn_copy_upload and the two ordering calls)
    def copy_upload(self, dst: "DeviceArray", host_ptr: int, nbytes: int) -> None:
        call("gbn_copy_upload", self.handle, dst.ptr, C.c_void_p(int(host_ptr)), int(nbytes))

    def copy_wait_compute(self) -> None:
        call("gbn_copy_wait_compute", self.handle)

    def compute_wait_copy(self) -> None:
        call("gbn_compute_wait_copy", self.handle)

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        call("gbn_ctx_get_stream", self.handle, C.byref(s))
        return s.value or 0

    def set_stream(self, stream: int | None) -> None:
        call("gbn_ctx_set_stream", self.handle, stream)

    def seed48(self, seed16v) -> None:
        arr = (C.c_ushort * 3)(*seed16v)
        call("gbn_ctx_seed48", self.handle, arr)

    def rand48(self) -> tuple[int, int, int]:
        arr = (C.c_ushort * 3)()
        call("gbn_ctx_get_rand48", self.handle, arr)
        return tuple(arr)

    def set_tuning(self, key: str, value: int) -> None:
        call("gbn_ctx_set_tuning", self.handle, key.encode(), int(value))

    def autotune(self, shapes, cache_path: str | None = None) -> None:
        """gbn_autotune over shapes [(W, H, F, C), ...]."""
        flat = np.ascontiguousarray(np.asarray(shapes, np.int32).reshape(-1, 4))
        call("gbn_autotune", self.handle, int(flat.shape[0]), flat.ctypes.data,
             cache_path.encode() if cache_path else None)

    def autotune_load(self, cache_path: str) -> None:
        call("gbn_autotune_load", self.handle, cache_path.encode())

    def tuning_for(self, W: int, H: int, F: int, Cc: int) -> tuple[int, int]:
        """(k1_coils_per_block, k2_ctas_per_sm) a run of this shape uses."""
        a, b = C.c_int(), C.c_int()
        call("gbn_autotune_lookup", self.handle, int(W), int(H), int(F), int(Cc), C.byref(a), C.byref(b))
        return a.value, b.value

    def launch_count(self) -> int:
        n = C.c_ulonglong()
        call("gbn_ctx_launch_count", self.handle, C.byref(n))
        return int(n.value)

    def profile(self, enable: bool) -> None:
        call("gbn_ctx_profile", self.handle, int(bool(enable)))

    def profile_reset(self) -> None:
        call("gbn_ctx_profile_reset", self.handle)

    def profile_read(self) -> dict[str, tuple[int, float]]:
        """{group: (launches, total ms)} of the event-profiled kernel groups."""
        out = {}
        for name, kind in _abi.PROFILE_KINDS.items():
            n, ms = C.c_ulonglong(), C.c_double()
            call("gbn_ctx_profile_read", self.handle, kind, C.byref(n), C.byref(ms))
            out[name] = (int(n.value), float(ms.value))
        return out


def supported_lengths() -> list[int]:
    buf = (C.c_int * 64)()
    n = _abi.lib().gbn_supported_lengths(buf, 64)
    return list(buf[:n])


def _ck(a: DeviceArray, dtype) -> int:
    if a.dtype != np.dtype(dtype):
        raise TypeError(f"expected {np.dtype(dtype)}, got {a.dtype}")
    return a.ptr


# operator entry points on device arrays --------------------------------------
def op_ttv(ctx: Context, direction: int, x: DeviceArray, out: DeviceArray) -> None:
    F, H, W = x.shape
    call("gbn_op_ttv", ctx.handle, direction, _ck(x, np.complex64), _ck(out, np.complex64), W, H, F)


def op_normalize(ctx: Context, x: DeviceArray, out: DeviceArray, mu: float) -> None:
    call("gbn_op_normalize", ctx.handle, _ck(x, np.complex64), _ck(out, np.complex64), x.size, float(mu))


def op_sensmul(ctx: Context, conjugate: bool, x: DeviceArray, S: DeviceArray, out: DeviceArray) -> None:
    F, Cc, H, W = out.shape
    in_coils = 1 if len(x.shape) == 4 else 0
    call("gbn_op_sensmul", ctx.handle, int(bool(conjugate)), _ck(x, np.complex64), in_coils,
         _ck(S, np.complex64), _ck(out, np.complex64), W, H, F, Cc)


def op_coilsum(ctx: Context, k: DeviceArray, out: DeviceArray) -> None:
    F, Cc, H, W = k.shape
    call("gbn_op_coilsum", ctx.handle, _ck(k, np.complex64), _ck(out, np.complex64), W, H, F, Cc)


def op_mask(ctx: Context, k: DeviceArray, mask: DeviceArray) -> None:
    F, Cc, H, W = k.shape
    call("gbn_op_mask", ctx.handle, _ck(k, np.complex64), _ck(mask, np.uint8), W, H, F, Cc)


def op_rowmask_to_pixelmask(ctx: Context, rowmask: DeviceArray, pixmask: DeviceArray) -> None:
    F, H, W = pixmask.shape
    call("gbn_op_rowmask_to_pixelmask", ctx.handle, _ck(rowmask, np.uint32), _ck(pixmask, np.uint8), W, H, F)


def op_abs(ctx: Context, x: DeviceArray, out: DeviceArray, squared: bool = False) -> None:
    call("gbn_op_abs2" if squared else "gbn_op_abs", ctx.handle, _ck(x, np.complex64),
         _ck(out, np.complex64), x.size)


def op_fft2(ctx: Context, direction: int, x: DeviceArray, out: DeviceArray) -> None:
    H, W = x.shape[-2:]
    batch = x.size // (H * W)
    call("gbn_op_fft2", ctx.handle, direction, _ck(x, np.complex64), _ck(out, np.complex64), W, H, batch)


def op_encode(ctx: Context, x: DeviceArray, S: DeviceArray, mask: DeviceArray, out: DeviceArray) -> None:
    F, Cc, H, W = out.shape
    call("gbn_op_encode", ctx.handle, _ck(x, np.complex64), _ck(S, np.complex64), _ck(mask, np.uint8),
         _ck(out, np.complex64), W, H, F, Cc)


def op_encode_adjoint(ctx: Context, k: DeviceArray, S: DeviceArray, out: DeviceArray) -> None:
    F, Cc, H, W = k.shape
    call("gbn_op_encode_adjoint", ctx.handle, _ck(k, np.complex64), _ck(S, np.complex64),
         _ck(out, np.complex64), W, H, F, Cc)


def simple_recon(ctx: Context, y: DeviceArray, S: DeviceArray, out: DeviceArray) -> None:
    F, Cc, H, W = y.shape
    call("gbn_simple_recon", ctx.handle, _ck(y, np.complex64), _ck(S, np.complex64),
         _ck(out, np.complex64), W, H, F, Cc)


def op_motion(ctx: Context, direction: int, x: DeviceArray, out: DeviceArray, xn: DeviceArray, xmesh: DeviceArray,
              bound_box) -> None:
    F, H, W = x.shape
    bb = (C.c_int * 4)(*[int(v) for v in bound_box])
    call("gbn_op_motion", ctx.handle, int(direction), _ck(x, np.complex64), _ck(out, np.complex64),
         _ck(xn, np.float32), _ck(xmesh, np.int32), bb, W, H, F)


def registration_params(W=1.0, flagW=True, radius=40, E=3, Dp=(4, 4), nmax=100, et=0.01, eh=0.005,
                        lambda_=(0.0, 0.005, 0.0, 0.5)) -> "_abi.RegistrationParams":
    """GroupwiseRegistration::InitParameters; defaults are tests/MRIRecon.cpp:121-129."""
    return _abi.RegistrationParams(float(W), int(bool(flagW)), int(radius), int(E), (C.c_int * 2)(*map(int, Dp)),
                                   int(nmax), float(et), float(eh), (C.c_float * 4)(*map(float, lambda_)))


def registration_info(N: int, F: int, params) -> dict:
    info = _abi.RegistrationInfo()
    call("gbn_registration_info_get", int(N), int(F), C.byref(params), C.byref(info))
    return dict(cp=info.cp, bound_box=list(info.bound_box), area=info.area)


def registration(ctx: Context, images: DeviceArray, params, T_init: DeviceArray | None = None) -> dict:
    """GroupwiseRegistration of images [F][N][N] complex (device).  Returns the
    control displacements T [2][F][cp][cp], the deformed mesh xn [2][F][N][N],
    the original mesh xmesh [2][N][N] (device arrays; the inputs of
    Problem.set_motion with bound_box), the metric per iteration and stats."""
    F, N, N2 = images.shape
    if N != N2:
        raise ValueError("square images only")
    info = registration_info(N, F, params)
    cp = info["cp"]
    T = ctx.empty((2, F, cp, cp), np.float32)
    xn = ctx.empty((2, F, N, N), np.float32)
    xmesh = ctx.empty((2, N, N), np.int32)
    H = np.zeros(params.nmax + 1, np.float32)
    st = _abi.RegistrationStats()
    call("gbn_registration_run", ctx.handle, _ck(images, np.complex64), N, F, C.byref(params),
         None if T_init is None else _ck(T_init, np.float32), T.ptr, xn.ptr, xmesh.ptr,
         H.ctypes.data, C.byref(st))
    stats = st.as_dict()
    stats["H_final"] = stats.pop("H")
    return dict(T=T, xn=xn, xmesh=xmesh, bound_box=info["bound_box"], H=H[:stats["iterations"] + 1],
                area=info["area"], cp=cp, **stats)


def op_rss(ctx: Context, k: DeviceArray, out: DeviceArray) -> None:
    F, Cc, H, W = k.shape
    call("gbn_op_rss", ctx.handle, _ck(k, np.complex64), _ck(out, np.complex64), W, H, F, Cc)


def simple_recon_sos(ctx: Context, y: DeviceArray, out: DeviceArray) -> None:
    F, Cc, H, W = y.shape
    call("gbn_simple_recon_sos", ctx.handle, _ck(y, np.complex64), _ck(out, np.complex64), W, H, F, Cc)


class Problem:
    """Solver workspace bound to device-resident y, S and pixel mask."""

    def __init__(self, ctx: Context, y: DeviceArray, S: DeviceArray, mask: DeviceArray):
        F, Cc, H, W = y.shape
        h = C.c_void_p()
        call("gbn_problem_create", ctx.handle, W, H, F, Cc, _ck(y, np.complex64), _ck(S, np.complex64),
             _ck(mask, np.uint8), C.byref(h))
        self.handle = h.value
        self.ctx, self.shape = ctx, (F, Cc, H, W)
        self._keep = (y, S, mask)
        ctx._children.add(self)

    def fit_rows(self, headroom_rows: int = 0) -> int:
        """Resize the row buffer to the rows the current y and mask keep plus
        headroom (gbn_problem_fit_rows); returns the kept rows."""
        g = C.c_int(0)
        call("gbn_problem_fit_rows", self.handle, int(headroom_rows), C.byref(g))
        return g.value

    def set_motion(self, xn: DeviceArray | None, xmesh: DeviceArray | None, bound_box=None) -> None:
        """Motion-compensated sparsity operator (gbn_problem_set_motion); the
        run then starts from the image already in its output buffer."""
        if xn is None:
            call("gbn_problem_set_motion", self.handle, None, None, None)
            self._motion = None
            return
        bb = (C.c_int * 4)(*[int(v) for v in bound_box])
        call("gbn_problem_set_motion", self.handle, _ck(xn, np.float32), _ck(xmesh, np.int32), bb)
        self._motion = (xn, xmesh)

    def run(self, params: NestaParams, out: DeviceArray, stats: bool = True) -> dict | None:
        st = NestaStats() if stats else None
        call("gbn_nesta_run", self.ctx.handle, self.handle, C.byref(params), _ck(out, np.complex64),
             C.byref(st) if st is not None else None)
        return st.as_dict() if st is not None else None

    def close(self) -> None:
        if self.handle:
            call("gbn_problem_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


PRECISION_FP32 = 0
PRECISION_MIXED = 1


class Batch:
    """Many reconstructions solved together (gbn_batch_*): problems of equal
    (W, H) share every solver launch; the whole solve can be captured into one
    CUDA graph and replayed."""

    def __init__(self, ctx: Context, problems: list[Problem], params: list[NestaParams] | NestaParams,
                 outputs: list[DeviceArray], precision: int = PRECISION_FP32):
        n = len(problems)
        if isinstance(params, NestaParams):
            params = [params] * n
        if len(params) != n or len(outputs) != n:
            raise ValueError("problems, params and outputs must have the same length")
        hp = (C.c_void_p * n)(*[p.handle for p in problems])
        pp = (NestaParams * n)(*params)
        op = (C.c_void_p * n)(*[_ck(o, np.complex64) for o in outputs])
        h = C.c_void_p()
        call("gbn_batch_create", ctx.handle, n, hp, pp, op, int(precision), C.byref(h))
        self.handle = h.value
        self.ctx, self.n = ctx, n
        self._keep = (problems, outputs)
        ctx._children.add(self)

    def capture(self) -> None:
        call("gbn_batch_capture", self.handle)

    def launch(self) -> None:
        call("gbn_batch_launch", self.handle)

    def groups(self) -> tuple[int, int]:
        """(groups, groups whose forward pass runs on the tensor cores)."""
        ng, ntc = C.c_int(0), C.c_int(0)
        call("gbn_batch_groups", self.handle, C.byref(ng), C.byref(ntc))
        return ng.value, ntc.value

    PATHS = {0: "three_pass", 1: "three_pass_tc", 2: "row_local", 3: "row_local_tc"}

    def group_info(self, g: int) -> dict:
        """W, H, member indices and the inner iteration ("three_pass",
        "three_pass_tc", "row_local", "row_local_tc") of group g."""
        W, H, n, path = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
        idx = (C.c_int * 64)()
        call("gbn_batch_group_info", self.handle, int(g), C.byref(W), C.byref(H), C.byref(n), idx, C.byref(path))
        return {"W": W.value, "H": H.value, "members": list(idx[:n.value]), "path": self.PATHS[path.value]}

    def stats(self, i: int) -> dict:
        st = NestaStats()
        call("gbn_batch_stats", self.handle, int(i), C.byref(st))
        return st.as_dict()

    def close(self) -> None:
        if self.handle:
            call("gbn_batch_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def nesta_params(lambda_i=1e-2, mu_f=3e-4, La=1.0, maxIntIter=4, tolVar=3e-4, verbose=1, maxIter=100,
                 stoptest=1, miniter=7) -> NestaParams:
    """NestaUp::LaunchParameters (NestaUp.hpp:67-83); defaults are tests/MRIRecon.cpp:105-114."""
    return NestaParams(float(lambda_i), float(mu_f), float(La), int(maxIntIter), float(tolVar), int(verbose),
                       int(maxIter), int(stoptest), int(miniter))


def nesta_run_host(ctx: Context, y: np.ndarray, S: np.ndarray, mask: np.ndarray, params: NestaParams,
                   out: np.ndarray | None = None) -> tuple[np.ndarray, dict]:
    """End-to-end reconstruction from host arrays (uploads, runs, downloads)."""
    F, Cc, H, W = y.shape
    y = np.ascontiguousarray(y, np.complex64)
    S = np.ascontiguousarray(S, np.complex64)
    mask = np.ascontiguousarray(mask, np.uint8)
    if out is None:
        out = np.empty((F, H, W), np.complex64)
    st = NestaStats()
    call("gbn_nesta_run_host", ctx.handle, W, H, F, Cc, y.ctypes.data, S.ctypes.data, mask.ctypes.data,
         C.byref(params), out.ctypes.data, C.byref(st))
    return out, st.as_dict()
