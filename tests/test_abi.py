"""The C ABI library loads, exports every function declared in include/gbn.h,
and reports argument errors through status codes (no GPU work here)."""
from __future__ import annotations

import ctypes as C
import os
import re

import pytest

from tests.conftest import ROOT


def _declared() -> list[str]:
    hdr = open(os.path.join(ROOT, "include", "gbn.h")).read()
    return re.findall(r"^GBN_API\s+[\w\s\*]+?\b(gbn_\w+)\s*\(", hdr, flags=re.M)


def test_header_declares_entry_points():
    names = _declared()
    assert len(names) >= 30
    for n in ("gbn_ctx_create", "gbn_nesta_run", "gbn_op_ttv", "gbn_op_fft2", "gbn_simple_recon"):
        assert n in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(built_lib):
    from opencliper_gb300 import _abi
    assert set(_declared()) <= set(_abi.SIGNATURES), set(_declared()) - set(_abi.SIGNATURES)


def test_version_and_lengths(built_lib):
    import opencliper_gb300 as g
    assert g.lib().gbn_version() == 1
    lens = g.supported_lengths()
    assert lens[0] == 8 and lens[-1] == 512 and len(lens) == 36
    from tests.test_nesta_gpu import LENGTHS
    assert lens == LENGTHS  # the list the every-length GPU tests walk
    for L in lens:
        n = L
        for p in (2, 3, 5, 7):
            while n % p == 0:
                n //= p
        assert n == 1 and L % 8 == 0


def test_null_arguments_are_rejected(built_lib):
    from opencliper_gb300 import _abi
    lib = _abi.lib()
    assert lib.gbn_op_ttv(None, 1, None, None, 8, 8, 2) == _abi.GBN_ERR_INVALID
    assert b"null" in lib.gbn_last_error_string()
    assert lib.gbn_ctx_create(0, None) == _abi.GBN_ERR_INVALID
    assert lib.gbn_nesta_run(None, None, None, None, None) == _abi.GBN_ERR_INVALID


def test_context_creation_fails_cleanly_without_gpu(built_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import opencliper_gb300 as g
    with pytest.raises(g.GbnError) as ei:
        g.Context(0)
    assert ei.value.code in (-1, -3)
