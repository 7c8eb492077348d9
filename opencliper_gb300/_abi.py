"""ctypes binding of libgbnesta.so (declarations in include/gbn.h).

The shared library is built in-tree by ``python -m opencliper_gb300.build``.
There is no fallback: when the library is missing or cannot be loaded, every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libgbnesta.so"

GBN_OK = 0
GBN_ERR_INVALID = -1
GBN_ERR_UNSUPPORTED = -2
GBN_ERR_CUDA = -3
GBN_ERR_NOMEM = -4

GBN_TTV_ADJOINT = 0
GBN_TTV_FORWARD = 1
GBN_FFT_FORWARD = -1
GBN_FFT_BACKWARD = 1
GBN_NOT_CONJUGATE = 0
GBN_CONJUGATE = 1

PROFILE_KINDS = {"fwd_cols": 0, "rows": 1, "inv_cols": 2, "setup": 3, "outer": 4, "iter": 5}


class GbnError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class NestaParams(C.Structure):
    _fields_ = [("lambda_i", C.c_float), ("mu_f", C.c_float), ("La", C.c_float),
                ("maxIntIter", C.c_uint), ("tolVar", C.c_float), ("verbose", C.c_int),
                ("maxIter", C.c_uint), ("stoptest", C.c_uint), ("miniter", C.c_uint)]


class NestaStats(C.Structure):
    _fields_ = [("normU", C.c_float), ("maxX", C.c_float), ("maxUX", C.c_float),
                ("lambda_", C.c_float), ("muf", C.c_float), ("mu0", C.c_float),
                ("mu_final", C.c_float), ("tolVar_final", C.c_float), ("fx_final", C.c_float),
                ("qp_final", C.c_float), ("inner_iters", C.c_int), ("normest_iters", C.c_int),
                ("kept_rows", C.c_int), ("status", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class RegistrationParams(C.Structure):
    """gbn_registration_params (GroupwiseRegistration::InitParameters)."""
    _fields_ = [("W", C.c_float), ("flagW", C.c_int), ("radius", C.c_int), ("E", C.c_int), ("Dp", C.c_int * 2),
                ("nmax", C.c_int), ("et", C.c_float), ("eh", C.c_float), ("lambda_", C.c_float * 4)]


class RegistrationInfo(C.Structure):
    _fields_ = [("cp", C.c_int), ("bound_box", C.c_int * 4), ("area", C.c_int)]


class RegistrationStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("H0", C.c_float), ("H", C.c_float), ("Wn", C.c_float),
                ("Tdif", C.c_float), ("status", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_vp = C.c_void_p
_i = C.c_int
_sz = C.c_size_t
_f = C.c_float

# name -> argtypes (all return int status unless listed in _RESTYPE)
SIGNATURES: dict[str, list] = {
    "gbn_last_error_string": [],
    "gbn_version": [],
    "gbn_supported_lengths": [C.POINTER(C.c_int), _i],
    "gbn_ctx_create": [_i, C.POINTER(_vp)],
    "gbn_ctx_destroy": [_vp],
    "gbn_ctx_get_stream": [_vp, C.POINTER(_vp)],
    "gbn_ctx_set_stream": [_vp, _vp],
    "gbn_ctx_sync": [_vp],
    "gbn_ctx_seed48": [_vp, C.POINTER(C.c_ushort)],
    "gbn_ctx_get_rand48": [_vp, C.POINTER(C.c_ushort)],
    "gbn_ctx_set_tuning": [_vp, C.c_char_p, _i],
    "gbn_ctx_launch_count": [_vp, C.POINTER(C.c_ulonglong)],
    "gbn_ctx_profile": [_vp, _i],
    "gbn_ctx_profile_read": [_vp, _i, C.POINTER(C.c_ulonglong), C.POINTER(C.c_double)],
    "gbn_ctx_profile_reset": [_vp],
    "gbn_alloc": [_vp, _sz, C.POINTER(_vp)],
    "gbn_free": [_vp, _vp],
    "gbn_upload": [_vp, _vp, _vp, _sz],
    "gbn_download": [_vp, _vp, _vp, _sz],
    "gbn_download_async": [_vp, _vp, _vp, _sz],
    "gbn_memset": [_vp, _vp, _i, _sz],
    "gbn_host_alloc": [_sz, C.POINTER(_vp)],
    "gbn_host_free": [_vp],
    "gbn_op_ttv": [_vp, _i, _vp, _vp, _i, _i, _i],
    "gbn_op_normalize": [_vp, _vp, _vp, _sz, _f],
    "gbn_op_sensmul": [_vp, _i, _vp, _i, _vp, _vp, _i, _i, _i, _i],
    "gbn_op_coilsum": [_vp, _vp, _vp, _i, _i, _i, _i],
    "gbn_op_mask": [_vp, _vp, _vp, _i, _i, _i, _i],
    "gbn_op_rowmask_to_pixelmask": [_vp, _vp, _vp, _i, _i, _i],
    "gbn_op_abs": [_vp, _vp, _vp, _sz],
    "gbn_op_abs2": [_vp, _vp, _vp, _sz],
    "gbn_op_fft2": [_vp, _i, _vp, _vp, _i, _i, _i],
    "gbn_op_encode": [_vp, _vp, _vp, _vp, _vp, _i, _i, _i, _i],
    "gbn_op_encode_adjoint": [_vp, _vp, _vp, _vp, _i, _i, _i, _i],
    "gbn_simple_recon": [_vp, _vp, _vp, _vp, _i, _i, _i, _i],
    "gbn_simple_recon_static": [_vp, _vp, _vp, _vp, _i, _i, _i, _i],
    "gbn_problem_create": [_vp, _i, _i, _i, _i, _vp, _vp, _vp, C.POINTER(_vp)],
    "gbn_problem_destroy": [_vp],
    "gbn_problem_set_motion": [_vp, _vp, _vp, _vp],
    "gbn_problem_fit_rows": [_vp, _i, _vp],
    "gbn_copy_upload": [_vp, _vp, _vp, _sz],
    "gbn_copy_wait_compute": [_vp],
    "gbn_compute_wait_copy": [_vp],
    "gbn_op_motion": [_vp, _i, _vp, _vp, _vp, _vp, _vp, _i, _i, _i],
    "gbn_registration_info_get": [_i, _i, C.POINTER(RegistrationParams), C.POINTER(RegistrationInfo)],
    "gbn_registration_run": [_vp, _vp, _i, _i, C.POINTER(RegistrationParams), _vp, _vp, _vp, _vp, _vp,
                             C.POINTER(RegistrationStats)],
    "gbn_nesta_run": [_vp, _vp, C.POINTER(NestaParams), _vp, C.POINTER(NestaStats)],
    "gbn_nesta_run_host": [_vp, _i, _i, _i, _i, _vp, _vp, _vp, C.POINTER(NestaParams), _vp,
                           C.POINTER(NestaStats)],
    "gbn_op_rss": [_vp, _vp, _vp, _i, _i, _i, _i],
    "gbn_simple_recon_sos": [_vp, _vp, _vp, _i, _i, _i, _i],
    "gbn_batch_create": [_vp, _i, C.POINTER(_vp), C.POINTER(NestaParams), C.POINTER(_vp), _i, C.POINTER(_vp)],
    "gbn_batch_launch": [_vp],
    "gbn_batch_capture": [_vp],
    "gbn_batch_stats": [_vp, _i, C.POINTER(NestaStats)],
    "gbn_batch_groups": [_vp, _vp, _vp],
    "gbn_batch_group_info": [_vp, _i, _vp, _vp, _vp, _vp, _vp],
    "gbn_batch_destroy": [_vp],
    "gbn_batch_run": [_vp, _i, C.POINTER(_vp), C.POINTER(NestaParams), C.POINTER(_vp), _i, C.POINTER(NestaStats)],
    "gbn_graph_capture": [_vp],
    "gbn_graph_replay": [_vp],
    "gbn_autotune": [_vp, _i, _vp, C.c_char_p],
    "gbn_autotune_load": [_vp, C.c_char_p],
    "gbn_autotune_lookup": [_vp, _i, _i, _i, _i, C.POINTER(_i), C.POINTER(_i)],
}
_RESTYPE = {"gbn_last_error_string": C.c_char_p}

_lib = None


def lib() -> C.CDLL:
    """Load libgbnesta.so once; raises when it is absent (no fallback path)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m opencliper_gb300.build`")
        L = C.CDLL(str(LIB_PATH))
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, C.c_int)
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != GBN_OK:
        msg = lib().gbn_last_error_string()
        raise GbnError(rc, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def exported_symbols() -> list[str]:
    return list(SIGNATURES)
