"""FP64 oracle: exact MixDom2 sufficient statistics (TEST INFRASTRUCTURE ONLY).

Part of the CPU oracle used by the test-suite to check the product's batched
implementation (``pairhmm.suffstats``); the product never imports it.

Restates, per pair in NumPy float64, the count restoration of
``models/exact_suffstats.py:31-103`` / ``models/exact_suffstats_batch.py:485-541``:

1. the fully exploded MixDom model with every null state explicit
   (``models/fully_exploded.py:21-235``): Start/End, the three top-level
   domain choosers, per-domain type choosers, fragment choosers, fragment-type
   states, the emitting states (in the collapsed chi's order), fragment ends
   and domain ends;
2. the null states eliminated, T_red = T_KK + T_KZ C T_ZK with
   C = (I - T_ZZ)^-1 (``models/elimination_steps.py:28-37``) -- here all null
   states in one step, which gives the same expected usages as the
   reference's six-step chain;
3. the collapsed counts restored on the exploded transitions by the
   ghost-usage formula of ``models/elimination_steps.py:40-124``;
4. the restored counts summed per parameter group
   (``models/exact_suffstats.py:106-227``).

Pinned against ``tests/golden/exact_suffstats.npz`` (the reference's own
outputs, ``tests/golden/make_golden_suffstats.py``).
"""
from __future__ import annotations

import numpy as np

from .models import tkf91_trans, S, M, I, D, E

KEYS = ('top_5x5', 'dom_M_5x5', 'dom_kappa', 'dom_1mkappa', 'ext', 'term', 'dom_w', 'frag_w')


class Exploded:
    """State indices of the fully exploded model for K domains, F fragments."""

    def __init__(self, K, F):
        self.K, self.F = K, F
        n = [0]

        def take(count):
            a = n[0]
            n[0] += count
            return a
        self.start, self.end = take(1), take(1)
        self.dom = take(3)                       # MatDom, InsDom, DelDom
        self.domtype = take(3 * K)               # [k][3]: Mat/Ins/Del domain type
        self.frag = take(5 * K)                  # [k][5]: MatFrag, InsFrag, DelFrag, IFrag, DFrag
        self.fragtype = take(5 * K * F)          # [k][f][5]
        self.emit = take(5 * K * F)              # [k][uv][f]: the collapsed chi's body order
        self.fragend = take(5 * K * F)           # [k][f][5]
        self.domend = take(3)                    # MatDomEnd, InsDomEnd, DelDomEnd
        self.N = n[0]
        self.kept = np.array([self.start, self.end] + list(range(self.emit, self.emit + 5 * K * F)))
        self.null = np.array([i for i in range(self.N) if i not in set(self.kept.tolist())])

    def domtype_i(self, k, x):
        return self.domtype + 3 * k + x

    def frag_i(self, k, x):
        return self.frag + 5 * k + x

    def fragtype_i(self, k, f, x):
        return self.fragtype + (k * self.F + f) * 5 + x

    def emit_i(self, k, x, f):
        return self.emit + k * 5 * self.F + x * self.F + f

    def fragend_i(self, k, f, x):
        return self.fragend + (k * self.F + f) * 5 + x


def build_exploded(main_ins, main_del, t, dom_ins, dom_del, dom_w, frag_w, ext):
    """The fully exploded transition matrix T [N_full, N_full] and its index map."""
    dom_ins, dom_del = np.asarray(dom_ins, float), np.asarray(dom_del, float)
    dom_w, frag_w = np.asarray(dom_w, float), np.asarray(frag_w, float)
    ext = np.asarray(ext, float)
    K, F = frag_w.shape
    if ext.ndim == 2:
        ext = np.stack([np.diag(ext[k]) for k in range(K)])
    X = Exploded(K, F)
    T = np.zeros((X.N, X.N))
    tau0 = tkf91_trans(main_ins, main_del, t)
    tauk = [tkf91_trans(dom_ins[k], dom_del[k], t) for k in range(K)]
    kap = dom_ins / dom_del
    # top level: Start and the domain ends choose the next domain mode or End
    for src, row in ((X.start, S), (X.domend, S), (X.domend + 1, S), (X.domend + 2, D)):
        for j, V in enumerate((M, I, D)):
            T[src, X.dom + j] = tau0[row, V]
        T[src, X.end] = tau0[row, E]
    for k in range(K):
        for j in range(3):
            T[X.dom + j, X.domtype_i(k, j)] = dom_w[k]
        # M-mode domain: its TKF91 start row, the phantom (empty) domain to the end
        for j, V in enumerate((M, I, D)):
            T[X.domtype_i(k, 0), X.frag_i(k, j)] = tauk[k][S, V]
        T[X.domtype_i(k, 0), X.domend] = tauk[k][S, E]
        # I- and D-mode domains: the kappa loop
        T[X.domtype_i(k, 1), X.frag_i(k, 3)] = kap[k]
        T[X.domtype_i(k, 1), X.domend + 1] = 1.0 - kap[k]
        T[X.domtype_i(k, 2), X.frag_i(k, 4)] = kap[k]
        T[X.domtype_i(k, 2), X.domend + 2] = 1.0 - kap[k]
        for f in range(F):
            notext = 1.0 - ext[k, f, :].sum()
            for x in range(5):
                T[X.frag_i(k, x), X.fragtype_i(k, f, x)] = frag_w[k, f]
                T[X.fragtype_i(k, f, x), X.emit_i(k, x, f)] = 1.0
                T[X.emit_i(k, x, f), X.fragend_i(k, f, x)] = 1.0
                for g in range(F):
                    T[X.fragend_i(k, f, x), X.fragtype_i(k, g, x)] = ext[k, f, g]
            # M-mode fragment ends continue the domain's TKF91 body rows
            for x, U in ((0, M), (1, I), (2, D)):
                for j, V in enumerate((M, I, D)):
                    T[X.fragend_i(k, f, x), X.frag_i(k, j)] = notext * tauk[k][U, V]
                T[X.fragend_i(k, f, x), X.domend] = notext * tauk[k][U, E]
            # I-/D-mode fragment ends: the kappa loop
            T[X.fragend_i(k, f, 3), X.frag_i(k, 3)] = notext * kap[k]
            T[X.fragend_i(k, f, 3), X.domend + 1] = notext * (1.0 - kap[k])
            T[X.fragend_i(k, f, 4), X.frag_i(k, 4)] = notext * kap[k]
            T[X.fragend_i(k, f, 4), X.domend + 2] = notext * (1.0 - kap[k])
    return T, X


def restore(n_red, T, X):
    """Exploded counts from collapsed counts by the ghost-usage formula."""
    Kp, Z = X.kept, X.null
    TKK, TKZ = T[np.ix_(Kp, Kp)], T[np.ix_(Kp, Z)]
    TZK, TZZ = T[np.ix_(Z, Kp)], T[np.ix_(Z, Z)]
    C = np.linalg.inv(np.eye(len(Z)) - TZZ)
    Tred = TKK + TKZ @ C @ TZK
    scale = np.where(np.abs(Tred) > 1e-30, n_red / np.where(np.abs(Tred) > 1e-30, Tred, 1.0), 0.0)
    H = C @ TZK
    Ct = TKZ @ C
    CtS = Ct.T @ scale
    n = np.zeros_like(T)
    n[np.ix_(Kp, Kp)] = scale * TKK
    n[np.ix_(Kp, Z)] = TKZ * (scale @ H.T)
    n[np.ix_(Z, Kp)] = TZK * CtS
    n[np.ix_(Z, Z)] = TZZ * (CtS @ H.T)
    return n, Tred


def extract(n, X):
    """Per-parameter-group sums of the restored counts."""
    K, F = X.K, X.F
    top = np.zeros((5, 5))
    for j, V in enumerate((M, I, D)):
        top[S, V] += n[X.start, X.dom + j]
    top[S, E] += n[X.start, X.end]
    for u, U in enumerate((M, I, D)):
        for j, V in enumerate((M, I, D)):
            top[U, V] += n[X.domend + u, X.dom + j]
        top[U, E] += n[X.domend + u, X.end]
    domM = np.zeros((K, 5, 5))
    kap = np.zeros(K)
    one_m_kap = np.zeros(K)
    ext = np.zeros((K, F, F))
    term = np.zeros((K, F))
    dom_w = np.zeros(K)
    frag_w = np.zeros((K, F))
    for k in range(K):
        for j, V in enumerate((M, I, D)):
            domM[k, S, V] = n[X.domtype_i(k, 0), X.frag_i(k, j)]
        domM[k, S, E] = n[X.domtype_i(k, 0), X.domend]
        kap[k] += n[X.domtype_i(k, 1), X.frag_i(k, 3)] + n[X.domtype_i(k, 2), X.frag_i(k, 4)]
        one_m_kap[k] += n[X.domtype_i(k, 1), X.domend + 1] + n[X.domtype_i(k, 2), X.domend + 2]
        for j in range(3):
            dom_w[k] += n[:, X.domtype_i(k, j)].sum()
        for f in range(F):
            for x, U in ((0, M), (1, I), (2, D)):
                fe = X.fragend_i(k, f, x)
                for j, V in enumerate((M, I, D)):
                    domM[k, U, V] += n[fe, X.frag_i(k, j)]
                domM[k, U, E] += n[fe, X.domend]
            kap[k] += n[X.fragend_i(k, f, 3), X.frag_i(k, 3)] + n[X.fragend_i(k, f, 4), X.frag_i(k, 4)]
            one_m_kap[k] += n[X.fragend_i(k, f, 3), X.domend + 1] + n[X.fragend_i(k, f, 4), X.domend + 2]
            for x in range(5):
                fe = X.fragend_i(k, f, x)
                e_tot = 0.0
                for g in range(F):
                    v = n[fe, X.fragtype_i(k, g, x)]
                    ext[k, f, g] += v
                    e_tot += v
                term[k, f] += n[fe, :].sum() - e_tot
                frag_w[k, f] += n[X.frag_i(k, x), X.fragtype_i(k, f, x)]
    return {'top_5x5': top, 'dom_M_5x5': domM, 'dom_kappa': kap, 'dom_1mkappa': one_m_kap,
            'ext': ext, 'term': term, 'dom_w': dom_w, 'frag_w': frag_w}


def exact_suffstats(n_chi, main_ins, main_del, t, dom_ins, dom_del, dom_w, frag_w, ext):
    """Per-pair exact sufficient statistics from collapsed counts n_chi [N, N]."""
    T, X = build_exploded(main_ins, main_del, t, dom_ins, dom_del, dom_w, frag_w, ext)
    n, _ = restore(np.asarray(n_chi, float), T, X)
    return extract(n, X)
