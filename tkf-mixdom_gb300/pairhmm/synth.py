"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: every configuration of the benchmark is
synthetic.  Parameters follow the stated laws (pi ~ Dirichlet(1*20),
exchangeabilities ~ LogNormal(0,1) symmetric and normalised to one expected
substitution per unit time, lambda ~ U(0.01,0.05), mu = lambda*U(1.05,1.5),
t ~ LogUniform(0.05,2), fragment extension r ~ U(0.3,0.9), Dirichlet(1)
weights and class distributions).  Ancestors are iid residues; descendants
are sampled by walking the pair HMM conditioned on the ancestor: M and D
moves consume the next ancestor residue and are only allowed while one is
left, End only once all are consumed, and the remaining moves are
renormalised -- the conditioning rule of the reference's simulator
(simulate/evolve.py:21-120), written here for any state space.  MixDom2
emissions pick the site class from its posterior given the ancestor residue.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

from . import models as pm

A = 20


def rand_Q_pi(rng, A_=A):
    """Reversible rate matrix with one expected substitution per unit time.
    Returns (Q, pi, S_exch) with Q[a,b] = S[a,b] pi[b]."""
    pi = rng.dirichlet(np.ones(A_))
    Sx = rng.lognormal(0.0, 1.0, size=(A_, A_))
    Sx = np.triu(Sx, 1)
    Sx = Sx + Sx.T
    Q = Sx * pi[None, :]
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(axis=1))
    rate = -np.sum(pi * np.diag(Q))
    return Q / rate, pi, Sx / rate


def mixdom2_params(rng, K, F, C):
    """A MixDom2 parameter dict with the reference's keys
    (train/likelihood.py:181-185): main_ins, main_del, t, dom_ins, dom_del,
    dom_weights, frag_weights, ext_rates (K,F), class_pis, class_S_exch,
    classdist."""
    cls = [rand_Q_pi(rng) for _ in range(C)]
    p = {
        'main_ins': float(rng.uniform(0.01, 0.05)),
        't': float(np.exp(rng.uniform(np.log(0.05), np.log(2.0)))),
        'dom_ins': rng.uniform(0.01, 0.05, K),
        'dom_weights': rng.dirichlet(np.ones(K)),
        'frag_weights': np.stack([rng.dirichlet(np.ones(F)) for _ in range(K)]),
        'ext_rates': rng.uniform(0.3, 0.9, (K, F)),
        'class_pis': np.stack([c[1] for c in cls]),
        'class_S_exch': np.stack([c[2] for c in cls]),
        'classdist': np.stack([[rng.dirichlet(np.ones(C)) for _ in range(F)] for _ in range(K)]),
    }
    p['main_del'] = p['main_ins'] * float(rng.uniform(1.05, 1.5))
    p['dom_del'] = p['dom_ins'] * rng.uniform(1.05, 1.5, K)
    return p


def tkf_params(rng, ext=None):
    Q, pi, _ = rand_Q_pi(rng)
    lam = float(rng.uniform(0.01, 0.05))
    p = {'ins_rate': lam, 'del_rate': lam * float(rng.uniform(1.05, 1.5)),
         't': float(np.exp(rng.uniform(np.log(0.05), np.log(2.0)))), 'Q': Q, 'pi': pi}
    if ext is not None:
        p['ext'] = ext
    return p


def walk_descendant(rng, x, chi, st, groups, emit_M_rows, emit_ins):
    """Sample a descendant of ancestor x by a conditioned pair-HMM walk.

    emit_M_rows(g, a) -> distribution over descendant residues for an M
    state of group g aligned to ancestor residue a; emit_ins(g) -> insert
    distribution of group g."""
    Lx = len(x)
    N = chi.shape[0]
    e_idx = int(np.argmax(st == pm.E))
    cur = 0
    pos = 0
    y = []
    cum = chi.cumsum(axis=1)
    for _ in range(10 * Lx + 1000):
        w = chi[cur].copy()
        if pos >= Lx:
            w[(st == pm.M) | (st == pm.D)] = 0.0
        else:
            w[e_idx] = 0.0
        w[(st == pm.S)] = 0.0
        tot = w.sum()
        if tot <= 0.0:
            break
        k = int(np.searchsorted(np.cumsum(w), rng.random() * tot, side='right'))
        k = min(k, N - 1)
        if k == e_idx:
            break
        g = groups[k]
        if st[k] == pm.M:
            pr = emit_M_rows(g, int(x[pos]))
            y.append(int(np.searchsorted(np.cumsum(pr), rng.random() * pr.sum(), side='right')))
            pos += 1
        elif st[k] == pm.I:
            pr = emit_ins(g)
            y.append(int(np.searchsorted(np.cumsum(pr), rng.random() * pr.sum(), side='right')))
        elif st[k] == pm.D:
            pos += 1
        cur = k
    del cum
    return np.minimum(np.asarray(y, dtype=np.int64), A - 1)


@dataclass
class Workload:
    """A batch of pairs with per-pair times and one parameter set."""
    name: str
    model: str                  # 'tkf91' | 'tkf92' | 'mixdom2'
    params: dict
    xs: list
    ys: list
    ts: np.ndarray
    K: int = 1
    F: int = 1
    C: int = 1
    meta: dict = field(default_factory=dict)

    @property
    def n_states(self):
        return 5 if self.model != 'mixdom2' else pm.mixdom_n_states(self.K, self.F)

    def cells(self):
        return np.array([(len(x) + 1) * (len(y) + 1) for x, y in zip(self.xs, self.ys)], np.int64)


def _lengths(rng, law, n):
    kind = law[0]
    if kind == 'uniform_int':
        return rng.integers(law[1], law[2] + 1, n)
    if kind == 'loguniform':
        return np.round(np.exp(rng.uniform(np.log(law[1]), np.log(law[2]), n))).astype(np.int64)
    if kind == 'around':
        c, frac = law[1], law[2]
        return rng.integers(int(c * (1 - frac)), int(c * (1 + frac)) + 1, n)
    raise ValueError(law)


def make_mixdom2_workload(name, K, F, C, n_pairs, law, seed=0):
    rng = np.random.default_rng(seed)
    p = mixdom2_params(rng, K, F, C)
    Lx = _lengths(rng, law, n_pairs)
    ts = np.exp(rng.uniform(np.log(0.05), np.log(2.0), n_pairs))
    st = pm.mixdom_state_types(K, F)
    groups = pm.mixdom_state_groups(K, F)
    cd = p['classdist'].reshape(K * F, C)
    cpi = p['class_pis']
    chis = pm.build_nested_trans(p['main_ins'], p['main_del'], torch.as_tensor(ts), p['dom_ins'],
                                 p['dom_del'], p['dom_weights'], p['frag_weights'], p['ext_rates']).numpy()
    csubs = pm.class_subs(p['class_S_exch'], cpi, torch.as_tensor(ts)).numpy()   # [P,C,A,A]
    anc_pi = (cd.mean(axis=0)[:, None] * cpi).sum(axis=0)
    xs, ys = [], []
    for b in range(n_pairs):
        x = rng.choice(A, size=int(Lx[b]), p=anc_pi / anc_pi.sum())

        def emit_M_rows(g, a, b=b):
            wc = cd[g] * cpi[:, a]
            wc = wc / wc.sum()
            return (wc[:, None] * csubs[b][:, a, :]).sum(axis=0)

        def emit_ins(g):
            return (cd[g][:, None] * cpi).sum(axis=0)
        y = walk_descendant(rng, x, chis[b], st.astype(np.int64), groups, emit_M_rows, emit_ins)
        xs.append(x.astype(np.int64))
        ys.append(y)
    return Workload(name, 'mixdom2', p, xs, ys, ts, K, F, C, {'law': law, 'seed': seed})


def make_tkf91_workload(name, n_pairs, law, seed=0):
    rng = np.random.default_rng(seed)
    p = tkf_params(rng)
    Lx = _lengths(rng, law, n_pairs)
    ts = np.exp(rng.uniform(np.log(0.05), np.log(2.0), n_pairs))
    st = np.array([pm.S, pm.M, pm.I, pm.D, pm.E])
    chis = pm.tkf91_trans(p['ins_rate'], p['del_rate'], torch.as_tensor(ts)).numpy()
    subs = pm.transition_matrix(p['Q'], torch.as_tensor(ts)).numpy()
    xs, ys = [], []
    for b in range(n_pairs):
        x = rng.choice(A, size=int(Lx[b]), p=p['pi'])
        y = walk_descendant(rng, x, chis[b], st, np.zeros(5, int),
                            lambda g, a, b=b: subs[b][a], lambda g: p['pi'])
        xs.append(x.astype(np.int64))
        ys.append(y)
    return Workload(name, 'tkf91', p, xs, ys, ts, meta={'law': law, 'seed': seed})


def _fast_walk(rng, x, chi, st, groups, m_cdf, i_cdf):
    """walk_descendant with precomputed cumulative tables (for long streams).

    m_cdf[g, a] is the cumulative descendant distribution of an M state of
    group g over ancestor residue a; i_cdf[g] the insert distribution."""
    Lx = len(x)
    N = chi.shape[0]
    e_idx = int(np.argmax(st == pm.E))
    w_open = chi.copy()
    w_open[:, e_idx] = 0.0
    w_open[:, st == pm.S] = 0.0
    w_end = chi.copy()
    w_end[:, (st == pm.M) | (st == pm.D) | (st == pm.S)] = 0.0
    c_open = np.cumsum(w_open, axis=1)
    c_end = np.cumsum(w_end, axis=1)
    u = rng.random(3 * (Lx + 50) * 4)
    k_u = 0
    cur, pos, y = 0, 0, []
    for _ in range(10 * Lx + 1000):
        c = c_open[cur] if pos < Lx else c_end[cur]
        if c[-1] <= 0.0:
            break
        if k_u + 2 >= u.size:
            u = rng.random(u.size)
            k_u = 0
        k = min(int(np.searchsorted(c, u[k_u] * c[-1], side='right')), N - 1)
        k_u += 1
        if k == e_idx:
            break
        g = groups[k]
        if st[k] == pm.M:
            cm = m_cdf[g, int(x[pos])]
            y.append(int(np.searchsorted(cm, u[k_u] * cm[-1], side='right')))
            k_u += 1
            pos += 1
        elif st[k] == pm.I:
            ci = i_cdf[g]
            y.append(int(np.searchsorted(ci, u[k_u] * ci[-1], side='right')))
            k_u += 1
        elif st[k] == pm.D:
            pos += 1
        cur = k
    return np.minimum(np.asarray(y, dtype=np.int64), A - 1)


SERVING_MODELS = (('tkf92', 'tkf92', None), ('mixdom2_k3f1c1', 'mixdom2', (3, 1, 1)),
                  ('mixdom2_k4f2c2', 'mixdom2', (4, 2, 2)))


def make_serving_stream(n_requests, rate=5000.0, law=('loguniform', 20, 2000), seed=0):
    """The serving workload: Poisson arrivals at `rate` requests/s of single
    pair E-step jobs, the model drawn uniformly from TKF92 (5 states) and
    MixDom2 with K*F = 3 (17 states) and K*F = 8 (42 states), ancestor
    lengths from `law`, per-request t ~ LogUniform(0.05, 2), descendants by
    the conditioned pair-HMM walk of each model.

    Returns (models, requests, offsets): models maps a name to (kind,
    params); requests is a list of (model name, x, y, t); offsets are the
    arrival times in seconds from the start."""
    rng = np.random.default_rng(seed)
    models = {}
    for name, kind, shape in SERVING_MODELS:
        if kind == 'tkf92':
            models[name] = (kind, tkf_params(rng, ext=float(rng.uniform(0.3, 0.9))))
        else:
            models[name] = (kind, mixdom2_params(rng, *shape))
    names = [m[0] for m in SERVING_MODELS]
    which = rng.integers(0, len(names), n_requests)
    Lx = _lengths(rng, law, n_requests)
    ts = np.exp(rng.uniform(np.log(0.05), np.log(2.0), n_requests))
    offsets = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    reqs = []
    for j in range(n_requests):
        name = names[which[j]]
        kind, p = models[name]
        t = torch.as_tensor([ts[j]], dtype=torch.float64)
        if kind == 'tkf92':
            st = np.array([pm.S, pm.M, pm.I, pm.D, pm.E])
            groups = np.zeros(5, np.int64)
            chi = pm.tkf92_trans(p['ins_rate'], p['del_rate'], t, p['ext'])[0].numpy()
            sub = pm.transition_matrix(p['Q'], t)[0].numpy()
            m_cdf = np.cumsum(sub, axis=1)[None]
            i_cdf = np.cumsum(p['pi'])[None]
            anc = p['pi']
        else:
            K, F = len(p['dom_ins']), p['frag_weights'].shape[1]
            C = p['class_pis'].shape[0]
            st = pm.mixdom_state_types(K, F).astype(np.int64)
            groups = pm.mixdom_state_groups(K, F)
            chi = pm.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'],
                                        p['dom_weights'], p['frag_weights'], p['ext_rates'])[0].numpy()
            cs = pm.class_subs(p['class_S_exch'], p['class_pis'], t)[0].numpy()        # [C,A,A]
            cd = p['classdist'].reshape(K * F, C)
            cpi = p['class_pis']
            wc = cd[:, :, None] * cpi[None, :, :]                                     # [G,C,A]
            wc = wc / wc.sum(axis=1, keepdims=True)
            rows = np.einsum('gca,cab->gab', wc, cs)                                  # [G,A,A]
            m_cdf = np.cumsum(rows, axis=2)
            i_cdf = np.cumsum((cd[:, :, None] * cpi[None]).sum(axis=1), axis=1)
            anc = (cd.mean(axis=0)[:, None] * cpi).sum(axis=0)
        x = rng.choice(A, size=int(Lx[j]), p=anc / anc.sum())
        y = _fast_walk(rng, x, chi, st, groups, m_cdf, i_cdf)
        reqs.append((name, x.astype(np.int64), y, float(ts[j])))
    return models, reqs, offsets


# The benchmark configurations (synthetic stand-ins with the stated shapes).
CONFIGS = {
    'tkf91_64pairs_len50-150': lambda seed=0: make_tkf91_workload(
        'tkf91_64pairs_len50-150', 64, ('uniform_int', 50, 150), seed),
    'mixdom2_k3f1c1_200pairs_len30-600': lambda seed=0: make_mixdom2_workload(
        'mixdom2_k3f1c1_200pairs_len30-600', 3, 1, 1, 200, ('loguniform', 30, 600), seed),
    'mixdom2_k4f2c2_32pairs_len200-1500': lambda seed=0: make_mixdom2_workload(
        'mixdom2_k4f2c2_32pairs_len200-1500', 4, 2, 2, 32, ('loguniform', 200, 1500), seed),
    'mixdom2_k8f4c4_64pairs_len2000': lambda seed=0: make_mixdom2_workload(
        'mixdom2_k8f4c4_64pairs_len2000', 8, 4, 4, 64, ('around', 2000, 0.1), seed),
}
