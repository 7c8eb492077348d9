"""drand48 as used by the power-method restart of NestaUp::myNormest
(src/processes/nesta/NestaUp.cpp:369-385) -- test infrastructure.

drand48 is the POSIX 48-bit linear congruential generator
X_{n+1} = (0x5DEECE66D * X_n + 0xB) mod 2^48, returning X_{n+1} / 2^48.  glibc's
state before any seeding is X_0 = 0x1234ABCD330E.  `libc_sequence` draws from
the C library itself (after resetting it with seed48 to that default state);
`lcg_sequence` is a vectorised restatement that the tests pin against it.
"""
from __future__ import annotations

import ctypes
import ctypes.util

import numpy as np

A = 0x5DEECE66D
C = 0xB
MASK = (1 << 48) - 1
DEFAULT_STATE = 0x1234ABCD330E


def state_to_seed16v(x: int) -> tuple[int, int, int]:
    return (x & 0xFFFF, (x >> 16) & 0xFFFF, (x >> 32) & 0xFFFF)


def seed16v_to_state(v) -> int:
    return int(v[0]) | (int(v[1]) << 16) | (int(v[2]) << 32)


def jump(k: int) -> tuple[int, int]:
    """(a, c) with X_{n+k} = a X_n + c mod 2^48."""
    ra, rc, ba, bc = 1, 0, A, C
    while k:
        if k & 1:
            ra, rc = (ba * ra) & MASK, (ba * rc + bc) & MASK
        ba, bc = (ba * ba) & MASK, (ba * bc + bc) & MASK
        k >>= 1
    return ra, rc


def lcg_sequence(n: int, state: int = DEFAULT_STATE) -> tuple[np.ndarray, int]:
    """n successive drand48() values (float64) and the state after them."""
    out = np.empty(n, np.uint64)
    blk = min(n, 4096)
    x = state
    for i in range(blk):
        x = (A * x + C) & MASK
        out[i] = x
    if n > blk:
        ja, jc = jump(blk)
        ja, jc, m = np.uint64(ja), np.uint64(jc), np.uint64(MASK)
        done = blk
        with np.errstate(over="ignore"):
            while done < n:
                k = min(blk, n - done)
                out[done:done + k] = (ja * out[done - blk:done - blk + k] + jc) & m
                done += k
    new_state = int(out[-1]) if n else state
    return out.astype(np.float64) * 2.0 ** -48, new_state


def libc_sequence(n: int, state: int = DEFAULT_STATE) -> tuple[np.ndarray, int]:
    """n values from the C library's drand48 after seed48(state)."""
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.drand48.restype = ctypes.c_double
    libc.seed48.argtypes = [ctypes.POINTER(ctypes.c_ushort)]
    libc.seed48.restype = ctypes.POINTER(ctypes.c_ushort)
    libc.seed48((ctypes.c_ushort * 3)(*state_to_seed16v(state)))
    vals = np.array([libc.drand48() for _ in range(n)], np.float64)
    # read the state back by re-seeding with it (seed48 returns the previous state)
    prev = libc.seed48((ctypes.c_ushort * 3)(*state_to_seed16v(DEFAULT_STATE)))
    new_state = seed16v_to_state([prev[0], prev[1], prev[2]])
    return vals, new_state
