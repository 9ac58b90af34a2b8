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
        i32 = ctypes.POINTER(ctypes.c_int32)
        lib.oracle_char_counts.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int8), i32, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, i32, i32, dp, dp, ctypes.c_double,
                                           dp, dp, dp]
        lib.oracle_char_counts.restype = None
        lib.oracle_set_threads.argtypes = [ctypes.c_int]
        lib.oracle_set_threads.restype = ctypes.c_int
        _L = lib
    return _L


def set_threads(n):
    """Host threads of the C oracle's anti-diagonal loops (1 = serial; the
    library's OpenMP default is every core).  Returns the number in use."""
    return int(_lib().oracle_set_threads(int(n)))


def forward_backward(log_trans, state_types, emit, forward_only=False, counts=None):
    """(log-likelihood, expected transitions (N, N) or None) for a log
    emission table emit (Lx+1, Ly+1, N).  With counts = (groups, G, x, y) a
    third value: the per-group character counts (cM [G,21,21], cI [G,21],
    cD [G,21]) of oracle.estep.char_count_tables."""
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
    if counts is None or forward_only:
        return float(ll), (None if forward_only else n)
    groups, G, x, y = counts
    gr = np.ascontiguousarray(np.asarray(groups, np.int32))
    xg = np.ascontiguousarray(np.concatenate([[0], np.asarray(x, np.int64)]).astype(np.int32))
    yg = np.ascontiguousarray(np.concatenate([[0], np.asarray(y, np.int64)]).astype(np.int32))
    emitting = np.isin(st, (1, 2, 3))
    if xg.size != Lx + 1 or yg.size != Ly + 1 or xg.min() < 0 or xg.max() > 20 or yg.min() < 0 or \
            yg.max() > 20 or gr.size != N or (emitting.any() and (gr[emitting].min() < 0 or gr[emitting].max() >= G)):
        raise ValueError('counts: sequences must match the table and hold 0..20, emitting groups 0..G-1')
    cM, cI, cD = np.zeros((G, 21, 21)), np.zeros((G, 21)), np.zeros((G, 21))
    i32 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    _lib().oracle_char_counts(N, st.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), i32(gr), int(G), Lx, Ly,
                              i32(xg), i32(yg), dp(F), dp(B), ll, dp(cM), dp(cI), dp(cD))
    return float(ll), n, (cM, cI, cD)
