"""FP64 oracle: 2D pair-HMM Viterbi (TEST INFRASTRUCTURE ONLY).

Part of the CPU oracle used by the test-suite to check the product's Viterbi
kernel (``pairhmm.api.viterbi_2d_batch``); the product never imports it.

Restates ``dp/hmm.py:1976-2040`` in NumPy float64: V[0,0,S] = 0, every
other entry NEG_INF until set; for each cell and each M / I / D state k the
best source s of V[pred(k)] + logchi[:, k] (the first maximum, as argmax),
plus the emission of _pair_hmm_emission (dp/hmm.py:617-625) with
log(pi + 1e-30) and log(P + 1e-30); the terminal maximum over
V[Lx, Ly] + logchi[:, E]; the path walked back from it.  Pinned against
``tests/golden/viterbi.npz`` (the reference's own outputs,
``tests/golden/make_golden_viterbi.py``).
"""
from __future__ import annotations

import numpy as np

from .models import S, M, I, D, E, NEG_INF


def viterbi_2d(log_trans, state_types, x, y, sub, pi):
    lt = np.asarray(log_trans, float)
    st = np.asarray(state_types)
    x, y = np.asarray(x, int), np.asarray(y, int)
    Lx, Ly, N = len(x), len(y), lt.shape[0]
    ls = np.log(np.asarray(sub, float) + 1e-30)
    lp = np.log(np.asarray(pi, float) + 1e-30)
    V = np.full((Lx + 1, Ly + 1, N), NEG_INF)
    V[0, 0, S] = 0.0
    TB = np.zeros((Lx + 1, Ly + 1, N, 3), int)
    for d in range(1, Lx + Ly + 1):
        for i in range(max(0, d - Ly), min(d, Lx) + 1):
            j = d - i
            xi, yj = x[max(i - 1, 0)] if Lx else 0, y[max(j - 1, 0)] if Ly else 0
            for k in range(N):
                t = st[k]
                if t == M and i > 0 and j > 0:
                    pi_, pj_, e = i - 1, j - 1, lp[xi] + ls[xi, yj]
                elif t == I and j > 0:
                    pi_, pj_, e = i, j - 1, lp[yj]
                elif t == D and i > 0:
                    pi_, pj_, e = i - 1, j, lp[xi]
                else:
                    continue
                sc = V[pi_, pj_] + lt[:, k]
                b = int(np.argmax(sc))
                V[i, j, k] = sc[b] + e
                TB[i, j, k] = (pi_, pj_, b)
    e_idx = int(np.argmax(st == E))
    fin = V[Lx, Ly] + lt[:, e_idx]
    best = int(np.argmax(fin))
    path = []
    ci, cj, ck = Lx, Ly, best
    while ci > 0 or cj > 0:
        path.append((ci, cj, ck))
        ci, cj, ck = (int(v) for v in TB[ci, cj, ck])
    path.append((0, 0, S))
    return float(fin[best]), path[::-1]
