"""FP64 oracle: 2D pair-HMM emissions and forward/backward (TEST INFRASTRUCTURE ONLY).

Log-space NumPy float64 restatement of the reference's 2D DP
(``python/tkfmixdom/jax/dp/hmm.py``).  Used only by tests, ``smoke()`` and
the CPU-baseline leg of ``bench.py``, as the FP64 comparison for the CUDA
path; the product never imports it.

The recursion is evaluated one anti-diagonal at a time, vectorised over the
cells of the diagonal, exactly as ``_forward_2d_core_diag``
(dp/hmm.py:1186-1292) and ``_backward_2d_core_diag`` (dp/hmm.py:1295-1437)
do; the per-cell maths is that of the cell-by-cell reference forms
``_forward_2d_core`` (dp/hmm.py:1120-1183) and ``_backward_2d_core``
(dp/hmm.py:1695-1772).  Tables are returned at the real (unpadded) size;
padding to geometric bins (dp/hmm.py:66-98) and masking it with NEG_INF
(dp/hmm.py:1827-1831) leaves every real-region value unchanged, which the
golden fixtures confirm.
"""
from __future__ import annotations

import numpy as np
from scipy.special import logsumexp

from .models import S, M, I, D, E, NEG_INF, safe_log

A_WILD = 21          # alphabet 20 + wildcard index 20 (dp/hmm.py:646-648)


# ------------------------------------------------------------ emissions
def _grid_chars(x, y):
    x = np.asarray(x, dtype=np.int64)
    y = np.asarray(y, dtype=np.int64)
    # row/col 0 use the dummy character 0 (dp/hmm.py:650-651)
    return np.concatenate([[0], x]), np.concatenate([[0], y])


def group_tables_tkf(sub, pi):
    """Linear per-group tables (G=1) of ``pair_hmm_emissions``
    (dp/hmm.py:628-670): log(P+1e-30), log(pi+1e-30), wildcard index 20 has
    probability 1.  Returns EM (1,21,21), EI (1,21), ED (1,21)."""
    sub = np.asarray(sub, float)
    pi = np.asarray(pi, float)
    lp = np.zeros(A_WILD)
    ls = np.zeros((A_WILD, A_WILD))
    lp[:20] = np.log(pi + 1e-30)
    ls[:20, :20] = np.log(sub + 1e-30)
    EM = np.exp(lp[:, None] + ls)
    EI = np.exp(lp)
    return EM[None], EI[None], EI[None].copy()


def group_tables_per_class(class_subs, class_pis, class_dist):
    """Linear per-(d,f) tables of ``pair_hmm_emissions_per_class``
    (dp/hmm.py:673-783): emit_g = log sum_c cd[g,c] pi_c P_c with
    max(.,1e-30) clamps and NEG_INF for cd == 0.  G = K*F groups, g = d*F+f."""
    cs = np.asarray(class_subs, float)
    cp = np.asarray(class_pis, float)
    cd = np.asarray(class_dist, float)
    K, F, C = cd.shape
    lcs = np.zeros((C, A_WILD, A_WILD))
    lcp = np.zeros((C, A_WILD))
    lcs[:, :20, :20] = np.log(np.maximum(cs, 1e-30))
    lcp[:, :20] = np.log(np.maximum(cp, 1e-30))
    lcd = safe_log(cd).reshape(K * F, C)
    lm = lcp[:, :, None] + lcs                                  # (C,21,21)
    EM = np.exp(logsumexp(lcd[:, :, None, None] + lm[None], axis=1))
    EI = np.exp(logsumexp(lcd[:, :, None] + lcp[None], axis=1))
    return EM, EI, EI.copy()


def group_tables_per_domain(sub_matrices, pis, K):
    """Per-domain tables of ``pair_hmm_emissions_per_domain``
    (dp/hmm.py:786-851): domain d uses (pi_d, P_d), clamps max(.,1e-30).
    G = K groups (one per domain)."""
    sm = np.asarray(sub_matrices, float)
    ps = np.asarray(pis, float)
    lp = np.zeros((K, A_WILD))
    ls = np.zeros((K, A_WILD, A_WILD))
    lp[:, :20] = np.log(np.maximum(ps, 1e-30))
    ls[:, :20, :20] = np.log(np.maximum(sm, 1e-30))
    EM = np.exp(lp[:, :, None] + ls)
    EI = np.exp(lp)
    return EM, EI, EI.copy()


def log_emission_table(state_types, groups, x, y, EM, EI, ED):
    """(Lx+1, Ly+1, N) log emission table from per-group tables: M states
    use EM[g, x_i, y_j], I states EI[g, y_j], D states ED[g, x_i], S/E 0
    (dp/hmm.py:653-669)."""
    xg, yg = _grid_chars(x, y)
    st = np.asarray(state_types)
    N = st.shape[0]
    out = np.zeros((xg.size, yg.size, N))
    with np.errstate(divide='ignore'):
        lEM, lEI, lED = np.log(EM), np.log(EI), np.log(ED)
    for k in range(N):
        g = groups[k]
        if st[k] == M:
            out[:, :, k] = lEM[g][xg[:, None], yg[None, :]]
        elif st[k] == I:
            out[:, :, k] = lEI[g][yg][None, :]
        elif st[k] == D:
            out[:, :, k] = lED[g][xg][:, None]
    out[~np.isfinite(out)] = NEG_INF
    return out


# ------------------------------------------------------------ forward / backward
def _lse_contract(pred, log_trans):
    """logsumexp_s pred[c, s] + log_trans[s, k] for a batch of cells."""
    return logsumexp(pred[:, :, None] + log_trans[None, :, :], axis=1)


def forward_table(log_trans, state_types, emit):
    """Forward table F (Lx+1, Ly+1, N) and log-likelihood.

    F[0,0,0] = 0 (index 0 is the start state, dp/hmm.py:1212); for M/I/D
    destination k, F[i,j,k] = logsumexp_s F[pred(i,j), s] + logT[s,k] +
    e[i,j,k] with pred M:(i-1,j-1), I:(i,j-1), D:(i-1,j); S/E destinations
    are NEG_INF off the origin (dp/hmm.py:1214-1247).  LL = logsumexp_s
    F[Lx,Ly,s] + logT[s,E] (dp/hmm.py:1291)."""
    lt = np.asarray(log_trans, float)
    st = np.asarray(state_types)
    Lx1, Ly1, N = emit.shape
    Lx, Ly = Lx1 - 1, Ly1 - 1
    isM, isI, isD = st == M, st == I, st == D
    Ftab = np.full((Lx1, Ly1, N), NEG_INF)
    Ftab[0, 0, 0] = 0.0
    for d in range(1, Lx + Ly + 1):
        i = np.arange(max(0, d - Ly), min(d, Lx) + 1)
        j = d - i
        mval = np.full((i.size, N), NEG_INF)
        ok = (i >= 1) & (j >= 1)
        if ok.any():
            mval[ok] = _lse_contract(Ftab[i[ok] - 1, j[ok] - 1], lt) + emit[i[ok], j[ok]]
        ival = np.full((i.size, N), NEG_INF)
        ok = j >= 1
        if ok.any():
            ival[ok] = _lse_contract(Ftab[i[ok], j[ok] - 1], lt) + emit[i[ok], j[ok]]
        dval = np.full((i.size, N), NEG_INF)
        ok = i >= 1
        if ok.any():
            dval[ok] = _lse_contract(Ftab[i[ok] - 1, j[ok]], lt) + emit[i[ok], j[ok]]
        cell = np.where(isM[None], mval, np.where(isI[None], ival,
                        np.where(isD[None], dval, NEG_INF)))
        Ftab[i, j] = cell
    e_idx = int(np.argmax(st == E))
    ll = float(logsumexp(Ftab[Lx, Ly] + lt[:, e_idx]))
    return ll, Ftab


def backward_table(log_trans, state_types, emit):
    """Backward table B (Lx+1, Ly+1, N): B[Lx,Ly,s] = logT[s,E]; elsewhere
    B[i,j,s] = logsumexp_k logT[s,k] + e[succ_k] + B[succ_k, k] over M/I/D
    destinations k with succ M:(i+1,j+1), I:(i,j+1), D:(i+1,j)
    (dp/hmm.py:1695-1772, 1317-1381)."""
    lt = np.asarray(log_trans, float)
    st = np.asarray(state_types)
    Lx1, Ly1, N = emit.shape
    Lx, Ly = Lx1 - 1, Ly1 - 1
    isM, isI, isD = st == M, st == I, st == D
    e_idx = int(np.argmax(st == E))
    Btab = np.full((Lx1, Ly1, N), NEG_INF)
    Btab[Lx, Ly] = lt[:, e_idx]
    for d in range(Lx + Ly - 1, -1, -1):
        i = np.arange(max(0, d - Ly), min(d, Lx) + 1)
        j = d - i
        parts = []
        for mask, di, dj in ((isM, 1, 1), (isI, 0, 1), (isD, 1, 0)):
            val = np.full((i.size, N), NEG_INF)
            ok = (i + di <= Lx) & (j + dj <= Ly)
            if ok.any():
                succ = emit[i[ok] + di, j[ok] + dj] + Btab[i[ok] + di, j[ok] + dj]
                succ = np.where(mask[None], succ, NEG_INF)
                val[ok] = logsumexp(lt[None, :, :] + succ[:, None, :], axis=2)
            parts.append(val)
        Btab[i, j] = logsumexp(np.stack(parts), axis=0)
    return Btab


def expected_transitions(log_trans, state_types, emit, Ftab, Btab, ll):
    """n[s,k] = sum over cells of exp(F[src,s] + logT[s,k] + e[dst,k] +
    B[dst,k] - LL) for M/I/D k, plus n[s,E] = exp(F[Lx,Ly,s] + logT[s,E] -
    LL) (dp/hmm.py:1940-1971)."""
    lt = np.asarray(log_trans, float)
    st = np.asarray(state_types)
    Lx1, Ly1, N = emit.shape
    isM, isI, isD = st == M, st == I, st == D
    n = np.zeros((N, N))
    for mask, di, dj in ((isM, 1, 1), (isI, 0, 1), (isD, 1, 0)):
        Fs = Ftab[:Lx1 - di, :Ly1 - dj].reshape(-1, N)
        W = (emit[di:, dj:] + Btab[di:, dj:]).reshape(-1, N)
        if Fs.shape[0] == 0:
            continue
        for k in np.nonzero(mask)[0]:
            lw = Fs + lt[None, :, k] + W[:, k][:, None] - ll
            n[:, k] += np.exp(lw).sum(axis=0)
    e_idx = int(np.argmax(st == E))
    n[:, e_idx] += np.exp(Ftab[Lx1 - 1, Ly1 - 1] + lt[:, e_idx] - ll)
    return n


def forward_backward(log_trans, state_types, emit, forward_only=False):
    """(LL, posteriors, expected_trans, F, B) at the real lattice size
    (dp/hmm.py:1834-1973)."""
    ll, Ftab = forward_table(log_trans, state_types, emit)
    if forward_only:
        return ll, None, None, Ftab, None
    Btab = backward_table(log_trans, state_types, emit)
    post = np.exp(Ftab + Btab - ll)
    n = expected_transitions(log_trans, state_types, emit, Ftab, Btab, ll)
    return ll, post, n, Ftab, Btab
