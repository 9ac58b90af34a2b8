"""FP64 oracle: 1D alignment-conditioned forward-backward (TEST INFRASTRUCTURE ONLY).

Part of the CPU oracle used by the test-suite to check the product's 1D
kernel (``pairhmm.api.forward_backward_1d_batch`` / ``estep_1d_mixdom2``);
the product never imports it.

Restates in NumPy float64, log space:
  * the alignment-constrained emissions of ``dp/hmm.py:854-1082``: a column
    of type M emits (anc, desc) through the M-type states' tables, I emits
    desc, D emits anc; states of another type (and S, E) get NEG_INF;
    character 20 is the wildcard with factor 1; MixDom2 mixes the classes
    per (domain, fragment) location (``pair_hmm_emissions_constrained_per_class``);
  * the forward-backward of ``dp/hmm.py:127-250, 471-607``: alpha_0 =
    logχ[init] + e_0; alpha_t[k] = logsumexp_s(alpha_{t-1}[s] + logχ[s,k]) + e_t[k];
    log P = logsumexp_k(alpha_{L-1}[k] + logχ[k,final]); beta_{L-1} =
    logχ[:,final]; expected transitions: the initial, interior and terminal
    transition posteriors; a length-0 alignment has log P = logχ[init,final].

Pinned against ``tests/golden/fb1d.npz`` (the reference's own outputs,
``tests/golden/make_golden_fb1d.py``).
"""
from __future__ import annotations

import numpy as np
from scipy.special import logsumexp

from .models import S, M, I, D, E, NEG_INF, safe_log


def constrained_emissions_per_class(state_types, cols, anc, desc, class_subs, class_pis, classdist, K, F):
    """(L, N) log emissions of an alignment under the MixDom2 class mixture."""
    st = np.asarray(state_types)
    N = st.size
    cs = np.asarray(class_subs, float)
    cp = np.asarray(class_pis, float)
    cd = np.asarray(classdist, float)
    C, A = cp.shape
    L = len(cols)
    out = np.full((L, N), NEG_INF)
    for s in range(2, N):
        body = s - 2
        d, f = body // (5 * F), (body % (5 * F)) % F
        w = cd[d, f]
        for l in range(L):
            col = int(cols[l])
            if col != st[s]:
                continue
            a, b = int(anc[l]), int(desc[l])
            pa = np.array([np.maximum(cp[c, a], 1e-30) if a < A else 1.0 for c in range(C)])
            pb = np.array([np.maximum(cp[c, b], 1e-30) if b < A else 1.0 for c in range(C)])
            if col == M:
                sub = np.array([np.maximum(cs[c, a, b], 1e-30) if (a < A and b < A) else 1.0 for c in range(C)])
                val = np.sum(w * pa * sub)
            elif col == I:
                val = np.sum(w * pb)
            else:
                val = np.sum(w * pa)
            out[l, s] = np.log(val) if val > 0 else NEG_INF
    return out


def forward_backward_1d(log_trans, log_emit, init_state=S, final_state=E):
    """(log P, posteriors (L, N), expected transitions (N, N)) of one alignment."""
    lt = np.asarray(log_trans, float)
    le = np.asarray(log_emit, float)
    L, N = le.shape if le.ndim == 2 else (0, lt.shape[0])
    if L == 0:
        n = np.zeros((N, N))
        n[init_state, final_state] = 1.0
        return lt[init_state, final_state], np.zeros((0, N)), n
    al = np.zeros((L, N))
    al[0] = lt[init_state] + le[0]
    for t in range(1, L):
        al[t] = logsumexp(al[t - 1][:, None] + lt, axis=0) + le[t]
    lp = logsumexp(al[L - 1] + lt[:, final_state])
    be = np.zeros((L, N))
    be[L - 1] = lt[:, final_state]
    for t in range(L - 2, -1, -1):
        be[t] = logsumexp(lt + le[t + 1][None, :] + be[t + 1][None, :], axis=1)
    post = np.exp(al + be - lp)
    n = np.zeros((N, N))
    for t in range(L - 1):
        n += np.exp(al[t][:, None] + lt + le[t + 1][None, :] + be[t + 1][None, :] - lp)
    n[:, final_state] += np.exp(al[L - 1] + lt[:, final_state] - lp)
    n[init_state, :] += np.exp(lt[init_state] + le[0] + be[0] - lp)
    return lp, post, n


def estep_1d(chi, state_types, cols, anc, desc, class_subs, class_pis, classdist, K, F, e_idx=1):
    le = constrained_emissions_per_class(state_types, cols, anc, desc, class_subs, class_pis, classdist, K, F)
    return forward_backward_1d(safe_log(chi), le, 0, e_idx)
