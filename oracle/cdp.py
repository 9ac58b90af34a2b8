"""FP64 oracle, C half (TEST INFRASTRUCTURE ONLY): the 2D forward-backward of
oracle/fb2d.c through ctypes, with the inputs oracle.dp takes.  Same results
as oracle.dp.forward_backward (checked in tests/test_oracle_c_cpu.py), an
order of magnitude faster; used by bench.py's CPU legs when it is built."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build_oracle import LIB

_L = None


def available():
    return os.path.exists(LIB)


def _lib():
    global _L
    if _L is None:
        lib = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        lib.oracle_fb2d.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int8), dp, ctypes.c_int, ctypes.c_int,
                                    dp, ctypes.c_int, dp, dp, dp, dp]
        lib.oracle_fb2d.restype = ctypes.c_double
        _L = lib
    return _L


def forward_backward(log_trans, state_types, emit, forward_only=False):
    """(log-likelihood, expected transitions (N, N) or None) for a log
    emission table emit (Lx+1, Ly+1, N)."""
    lt = np.ascontiguousarray(np.asarray(log_trans, np.float64))
    st = np.ascontiguousarray(np.asarray(state_types, np.int8))
    em = np.ascontiguousarray(np.asarray(emit, np.float64))
    Lx, Ly, N = em.shape[0] - 1, em.shape[1] - 1, em.shape[2]
    if lt.shape != (N, N) or st.size != N:
        raise ValueError('log_trans (N, N), state_types (N,) and emit (Lx+1, Ly+1, N) disagree')
    F = np.empty_like(em)
    B = np.empty(0 if forward_only else em.size, np.float64)
    n = np.zeros((N, N))
    tmp = np.empty(max(N, 1), np.float64)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    ll = _lib().oracle_fb2d(N, st.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), dp(lt), Lx, Ly, dp(em),
                            int(bool(forward_only)), dp(F), dp(B) if B.size else None, dp(n), dp(tmp))
    return float(ll), (None if forward_only else n)
