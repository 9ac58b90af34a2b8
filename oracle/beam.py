"""FP64 oracle: beam-pruned pair-HMM forward-backward (TEST INFRASTRUCTURE ONLY).

Part of the CPU oracle the test-suite checks the product's beam path against;
the product never imports it.

Restates ``dp/hmm_beam.py`` in NumPy float64, log space:
  * ``msa_to_envelope`` (hmm_beam.py:22-82): cell (i, j) is in the envelope
    when j lies within band_width of the y range of the guide points whose
    i is within band_width of i; (0, 0) and (Lx, Ly) always are;
  * ``beam_forward_2d`` (hmm_beam.py:85-203): cells in anti-diagonal order,
    cells off the envelope skipped (NEG_INF); F[i,j,k] = lse_s(F[pred,s] +
    logT[s,k]) + emission, the lse taken as NEG_INF when its maximum is at
    most NEG_INF + 100; then every state below max_k F[i,j,k] - beam_log_width
    set to NEG_INF; emissions log max(pi, 1e-30) and log max(P, 1e-30);
  * ``beam_forward_backward_2d`` (hmm_beam.py:206-318): the backward only on
    cells the pruned forward left active (any state above NEG_INF + 100),
    from active successors, for every state of the cell; posteriors
    exp(min(F + B - log P, 0)) on active cells, 0 elsewhere;
  * ``beam_viterbi_2d`` (hmm_beam.py:397-490): the Viterbi recursion on the
    envelope, a state whose cell or predecessor cell lies outside keeping
    NEG_INF and the pointer (0, 0, S).

Pinned against ``tests/golden/beam.npz`` (the reference's own outputs,
``tests/golden/make_golden_beam.py``).
"""
from __future__ import annotations

import numpy as np

from .models import M, I, D, E, NEG_INF


def msa_to_envelope(x_len, y_len, msa_x_row, msa_y_row, band_width, gap_token=-1):
    pts = [(0, 0)]
    xi = yj = 0
    for a, b in zip(np.asarray(msa_x_row), np.asarray(msa_y_row)):
        xi += int(a) != gap_token
        yj += int(b) != gap_token
        pts.append((xi, yj))
    pts.append((x_len, y_len))
    pts = np.array(pts)
    env = np.zeros((x_len + 1, y_len + 1), bool)
    for i in range(x_len + 1):
        near = np.abs(pts[:, 0] - i) <= band_width
        lo = pts[near, 1].min() if near.any() else y_len
        hi = pts[near, 1].max() if near.any() else 0
        env[i, max(0, lo - band_width):min(y_len, hi + band_width) + 1] = True
    env[0, 0] = True
    env[x_len, y_len] = True
    return env


def _emission_table(state_types, x, y, sub, pi):
    st = np.asarray(state_types)
    ls = np.log(np.maximum(np.asarray(sub, float), 1e-30))
    lp = np.log(np.maximum(np.asarray(pi, float), 1e-30))
    xg = np.concatenate([[0], np.asarray(x, int)])
    yg = np.concatenate([[0], np.asarray(y, int)])
    em = np.zeros((xg.size, yg.size, st.size))
    for k in range(st.size):
        if st[k] == M:
            em[:, :, k] = lp[xg][:, None] + ls[xg[:, None], yg[None, :]]
        elif st[k] == I:
            em[:, :, k] = lp[yg][None, :]
        elif st[k] == D:
            em[:, :, k] = lp[xg][:, None]
    return em


def _lse(v):
    m = np.max(v)
    return m + np.log(np.sum(np.exp(v - m))) if m > NEG_INF + 100 else NEG_INF


def beam_forward(log_trans, state_types, x, y, sub, pi, beam_log_width=np.inf, envelope=None):
    """(log P, F (Lx+1, Ly+1, N), number of cells computed)."""
    lt = np.asarray(log_trans, float)
    st = np.asarray(state_types)
    em = _emission_table(st, x, y, sub, pi)
    Lx, Ly, N = em.shape[0] - 1, em.shape[1] - 1, st.size
    F = np.full((Lx + 1, Ly + 1, N), NEG_INF)
    F[0, 0, 0] = 0.0
    n_cells = 0
    for d in range(1, Lx + Ly + 1):
        for i in range(max(0, d - Ly), min(d, Lx) + 1):
            j = d - i
            if envelope is not None and not envelope[i, j]:
                continue
            n_cells += 1
            for k in range(N):
                if st[k] == M and i > 0 and j > 0:
                    pred = F[i - 1, j - 1]
                elif st[k] == I and j > 0:
                    pred = F[i, j - 1]
                elif st[k] == D and i > 0:
                    pred = F[i - 1, j]
                else:
                    continue
                F[i, j, k] = _lse(pred + lt[:, k]) + em[i, j, k]
            if np.isfinite(beam_log_width):
                mx = F[i, j].max()
                if mx > NEG_INF + 100:
                    F[i, j, F[i, j] < mx - beam_log_width] = NEG_INF
    e_idx = int(np.argmax(st == E))
    return _lse(F[Lx, Ly] + lt[:, e_idx]), F, n_cells


def beam_forward_backward(log_trans, state_types, x, y, sub, pi, beam_log_width=np.inf, envelope=None):
    """(log P, posteriors (Lx+1, Ly+1, N), F)."""
    lt = np.asarray(log_trans, float)
    st = np.asarray(state_types)
    lp, F, _ = beam_forward(lt, st, x, y, sub, pi, beam_log_width, envelope)
    Lx, Ly, N = F.shape[0] - 1, F.shape[1] - 1, st.size
    if lp <= NEG_INF + 100:
        return lp, np.zeros_like(F), F
    em = _emission_table(st, x, y, sub, pi)
    active = np.any(F > NEG_INF + 100, axis=2)
    e_idx = int(np.argmax(st == E))
    B = np.full_like(F, NEG_INF)
    B[Lx, Ly] = lt[:, e_idx]
    step = {M: (1, 1), I: (0, 1), D: (1, 0)}
    for d in range(Lx + Ly, 0, -1):
        for i in range(max(0, d - Ly), min(d, Lx) + 1):
            j = d - i
            if not active[i, j]:
                continue
            terms = []
            for s in range(N):
                if st[s] not in step:
                    continue
                ni, nj = i + step[st[s]][0], j + step[st[s]][1]
                if ni > Lx or nj > Ly or not active[ni, nj]:
                    continue
                terms.append(lt[:, s] + em[ni, nj, s] + B[ni, nj, s])
            if terms:
                T = np.stack(terms, axis=1)                       # [k, successor]
                tot = np.array([_lse(T[k]) for k in range(N)])
                cur = B[i, j]
                both = (cur > NEG_INF + 100) & (tot > NEG_INF + 100)
                B[i, j] = np.where(both, np.logaddexp(cur, tot), np.where(tot > NEG_INF + 100, tot, cur))
    post = np.zeros_like(F)
    post[active] = np.exp(np.minimum(F[active] + B[active] - lp, 0.0))
    return lp, post, F


def beam_viterbi(log_trans, state_types, x, y, sub, pi, envelope=None):
    """(log P of the best path, path [(i, j, state), ...]) of beam_viterbi_2d
    (hmm_beam.py:397-490): a state whose cell or predecessor cell is outside
    the envelope keeps NEG_INF and the pointer (0, 0, S); first maximum wins."""
    lt = np.asarray(log_trans, float)
    st = np.asarray(state_types)
    em = _emission_table(st, x, y, sub, pi)
    Lx, Ly, N = em.shape[0] - 1, em.shape[1] - 1, st.size
    V = np.full((Lx + 1, Ly + 1, N), NEG_INF)
    V[0, 0, 0] = 0.0
    TB = np.zeros((Lx + 1, Ly + 1, N, 3), np.int64)
    step = {M: (1, 1), I: (0, 1), D: (1, 0)}
    for d in range(1, Lx + Ly + 1):
        for i in range(max(0, d - Ly), min(d, Lx) + 1):
            j = d - i
            if envelope is not None and not envelope[i, j]:
                continue
            for k in range(N):
                if st[k] not in step:
                    continue
                pi_, pj_ = i - step[st[k]][0], j - step[st[k]][1]
                if pi_ < 0 or pj_ < 0:
                    continue
                if envelope is not None and not envelope[pi_, pj_]:
                    continue
                sc = V[pi_, pj_] + lt[:, k]
                b = int(np.argmax(sc))
                V[i, j, k] = sc[b] + em[i, j, k]
                TB[i, j, k] = (pi_, pj_, b)
    e_idx = int(np.argmax(st == E))
    fs = V[Lx, Ly] + lt[:, e_idx]
    ck = int(np.argmax(fs))
    path, ci, cj = [], Lx, Ly
    while ci > 0 or cj > 0:
        path.append((ci, cj, ck))
        ci, cj, ck = (int(v) for v in TB[ci, cj, ck])
    path.append((0, 0, 0))
    return float(fs[int(np.argmax(fs))]), path[::-1]
