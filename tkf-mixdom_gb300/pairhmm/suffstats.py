"""Exact MixDom2 sufficient statistics from collapsed E-step counts, batched
over pairs in float64 on the device (the E-step epilogue of
``models/exact_suffstats_batch.py:485-541``).

The collapsed pair HMM's chi is the null elimination of a fully exploded
model in which every transition carries one parameter factor
(``models/fully_exploded.py:21-235``: domain and fragment choosers, fragment
ends, domain ends).  Given the E-step's expected collapsed transition counts
n_chi, the expected usage of every exploded transition follows from the
ghost-usage formula of ``models/elimination_steps.py:40-124``; summing those
usages per parameter group gives the statistics of closed-form M-steps
(``models/exact_suffstats.py:106-227``).  Here all null states are
eliminated in one step, C = (I - T_ZZ)^-1 per pair, which yields the same
expected usages as the reference's six-step chain; the exploded matrix is
assembled on the host (float64, vectorised over pairs) and the inverse, the
restoration and the grouped sums run as batched torch operations on the
counts' device.
"""
from __future__ import annotations

import functools

import numpy as np
import torch

S, M, I, D, E = 0, 1, 2, 3, 4
F64 = torch.float64
KEYS = ('top_5x5', 'dom_M_5x5', 'dom_kappa', 'dom_1mkappa', 'ext', 'term', 'dom_w', 'frag_w')


class _Layout:
    """Indices of the exploded model's states for K domains and F fragments:
    Start, End, 3 domain choosers, 3K domain-type states, 5K fragment
    choosers, 5KF fragment-type states, 5KF emitting states (the collapsed
    chi's body order: domain, compound type, fragment), 5KF fragment ends,
    3 domain ends."""

    def __init__(self, K, F):
        self.K, self.F = K, F
        self.start, self.end, self.dom = 0, 1, 2
        self.domtype = 5
        self.frag = self.domtype + 3 * K
        self.fragtype = self.frag + 5 * K
        self.emit = self.fragtype + 5 * K * F
        self.fragend = self.emit + 5 * K * F
        self.domend = self.fragend + 5 * K * F
        self.N = self.domend + 3
        kept = [self.start, self.end] + list(range(self.emit, self.emit + 5 * K * F))
        ks = set(kept)
        self.kept = np.array(kept)
        self.null = np.array([i for i in range(self.N) if i not in ks])

    def dt(self, k, x):
        return self.domtype + 3 * k + x

    def fr(self, k, x):
        return self.frag + 5 * k + x

    def ft(self, k, f, x):
        return self.fragtype + (k * self.F + f) * 5 + x

    def em(self, k, x, f):
        return self.emit + k * 5 * self.F + x * self.F + f

    def fe(self, k, f, x):
        return self.fragend + (k * self.F + f) * 5 + x


def _tkf91(lam, mu, t):
    """[..., 5, 5] TKF91 matrices, float64 NumPy, broadcasting (core/params.py:29-55)."""
    lam, mu, t = np.broadcast_arrays(np.asarray(lam, float), np.asarray(mu, float), np.asarray(t, float))
    s = mu * t
    a = np.exp(-s)
    eta = np.exp(-lam * t)
    k = lam / mu
    near = np.abs(1.0 - k) < 1e-4
    with np.errstate(divide='ignore', invalid='ignore'):
        den = mu * eta - lam * a
        b = np.where(np.abs(den) < 1e-30, 0.0, lam * (eta - a) / np.where(np.abs(den) < 1e-30, 1.0, den))
        b = np.where(near, s / (1.0 + s), b)
        Phi = 1.0 - a
        g_gen = np.where(np.abs(Phi) < 1e-30, 0.0, 1.0 - mu * b / (lam * np.maximum(Phi, 1e-30)))
        phi = np.where(s < 1e-10, 1.0 - s / 2.0, Phi / np.maximum(s, 1e-30))
        g = np.where(near, 1.0 - 1.0 / ((1.0 + s) * phi), g_gen)
    z = np.zeros_like(a)
    row = np.stack([z, (1 - b) * k * a, b, (1 - b) * k * (1 - a), (1 - b) * (1 - k)], -1)
    rowD = np.stack([z, (1 - g) * k * a, g, (1 - g) * k * (1 - a), (1 - g) * (1 - k)], -1)
    return np.stack([row, row, row, rowD, np.zeros_like(row)], -2)


def _exploded(main_ins, main_del, t, dom_ins, dom_del, dom_w, frag_w, ext, L):
    """T [B, N_full, N_full] of the exploded model (models/fully_exploded.py:21-235)."""
    K, F = L.K, L.F
    B = t.shape[0]
    T = np.zeros((B, L.N, L.N))
    tau0 = _tkf91(main_ins, main_del, t)                      # [B,5,5]
    tauk = _tkf91(dom_ins[None, :], dom_del[None, :], t[:, None])   # [B,K,5,5]
    kap = dom_ins / dom_del
    for src, row in ((L.start, S), (L.domend, S), (L.domend + 1, S), (L.domend + 2, D)):
        for j, V in enumerate((M, I, D)):
            T[:, src, L.dom + j] = tau0[:, row, V]
        T[:, src, L.end] = tau0[:, row, E]
    for k in range(K):
        for j, V in enumerate((M, I, D)):
            T[:, L.dom + j, L.dt(k, j)] = dom_w[k]
            T[:, L.dt(k, 0), L.fr(k, j)] = tauk[:, k, S, V]
        T[:, L.dt(k, 0), L.domend] = tauk[:, k, S, E]
        T[:, L.dt(k, 1), L.fr(k, 3)] = kap[k]
        T[:, L.dt(k, 1), L.domend + 1] = 1.0 - kap[k]
        T[:, L.dt(k, 2), L.fr(k, 4)] = kap[k]
        T[:, L.dt(k, 2), L.domend + 2] = 1.0 - kap[k]
        for f in range(F):
            notext = 1.0 - ext[k, f, :].sum()
            for x in range(5):
                T[:, L.fr(k, x), L.ft(k, f, x)] = frag_w[k, f]
                T[:, L.ft(k, f, x), L.em(k, x, f)] = 1.0
                T[:, L.em(k, x, f), L.fe(k, f, x)] = 1.0
                for g in range(F):
                    T[:, L.fe(k, f, x), L.ft(k, g, x)] = ext[k, f, g]
            for x, U in ((0, M), (1, I), (2, D)):
                for j, V in enumerate((M, I, D)):
                    T[:, L.fe(k, f, x), L.fr(k, j)] = notext * tauk[:, k, U, V]
                T[:, L.fe(k, f, x), L.domend] = notext * tauk[:, k, U, E]
            T[:, L.fe(k, f, 3), L.fr(k, 3)] = notext * kap[k]
            T[:, L.fe(k, f, 3), L.domend + 1] = notext * (1.0 - kap[k])
            T[:, L.fe(k, f, 4), L.fr(k, 4)] = notext * kap[k]
            T[:, L.fe(k, f, 4), L.domend + 2] = notext * (1.0 - kap[k])
    return T


@functools.lru_cache(maxsize=32)
def _plan(K, F):
    """The layout and the grouped-sum recipe: output slot o receives
    w * v[src] for each (o, src, w), v = [n_full flattened, row sums, column sums]."""
    L = _Layout(K, F)
    N = L.N
    outs = {}   # name -> (shape, offset)
    o = 0
    for name, shape in (('top_5x5', (5, 5)), ('dom_M_5x5', (K, 5, 5)), ('dom_kappa', (K,)),
                        ('dom_1mkappa', (K,)), ('ext', (K, F, F)), ('term', (K, F)), ('dom_w', (K,)),
                        ('frag_w', (K, F))):
        outs[name] = (shape, o)
        o += int(np.prod(shape))
    recipe = []

    def add(name, at, src, w=1.0):
        shape, off = outs[name]
        recipe.append((off + int(np.ravel_multi_index(at, shape)), src, w))
    cell = lambda a, b: a * N + b
    row = lambda a: N * N + a
    col = lambda b: N * N + N + b
    for j, V in enumerate((M, I, D)):
        add('top_5x5', (S, V), cell(L.start, L.dom + j))
    add('top_5x5', (S, E), cell(L.start, L.end))
    for u, U in enumerate((M, I, D)):
        for j, V in enumerate((M, I, D)):
            add('top_5x5', (U, V), cell(L.domend + u, L.dom + j))
        add('top_5x5', (U, E), cell(L.domend + u, L.end))
    for k in range(K):
        for j, V in enumerate((M, I, D)):
            add('dom_M_5x5', (k, S, V), cell(L.dt(k, 0), L.fr(k, j)))
            add('dom_w', (k,), col(L.dt(k, j)))
        add('dom_M_5x5', (k, S, E), cell(L.dt(k, 0), L.domend))
        add('dom_kappa', (k,), cell(L.dt(k, 1), L.fr(k, 3)))
        add('dom_kappa', (k,), cell(L.dt(k, 2), L.fr(k, 4)))
        add('dom_1mkappa', (k,), cell(L.dt(k, 1), L.domend + 1))
        add('dom_1mkappa', (k,), cell(L.dt(k, 2), L.domend + 2))
        for f in range(F):
            for x, U in ((0, M), (1, I), (2, D)):
                for j, V in enumerate((M, I, D)):
                    add('dom_M_5x5', (k, U, V), cell(L.fe(k, f, x), L.fr(k, j)))
                add('dom_M_5x5', (k, U, E), cell(L.fe(k, f, x), L.domend))
            add('dom_kappa', (k,), cell(L.fe(k, f, 3), L.fr(k, 3)))
            add('dom_kappa', (k,), cell(L.fe(k, f, 4), L.fr(k, 4)))
            add('dom_1mkappa', (k,), cell(L.fe(k, f, 3), L.domend + 1))
            add('dom_1mkappa', (k,), cell(L.fe(k, f, 4), L.domend + 2))
            for x in range(5):
                add('term', (k, f), row(L.fe(k, f, x)))
                for g in range(F):
                    add('ext', (k, f, g), cell(L.fe(k, f, x), L.ft(k, g, x)))
                    add('term', (k, f), cell(L.fe(k, f, x), L.ft(k, g, x)), -1.0)
                add('frag_w', (k, f), cell(L.fr(k, x), L.ft(k, f, x)))
    dst = np.array([r[0] for r in recipe], np.int64)
    src = np.array([r[1] for r in recipe], np.int64)
    w = np.array([r[2] for r in recipe], np.float64)
    return L, outs, o, dst, src, w


def exact_suffstats_batch(n_chi_stack, main_ins, main_del, t_array, dom_ins, dom_del, dom_weights,
                          frag_weights, ext_rates):
    """Per-pair exact MixDom2 sufficient statistics (models/exact_suffstats_batch.py:485-541).

    n_chi_stack: [B, N, N] collapsed expected transition counts (a torch
    tensor -- the E-step's n_trans -- or an array); t_array [B] per-pair
    times; the other parameters shared.  Returns the reference's dict with a
    leading B axis: top_5x5 [B,5,5], dom_M_5x5 (a list of K [B,5,5]),
    dom_kappa / dom_1mkappa / dom_w [B,K], ext [B,K,F,F], term [B,K,F],
    frag_w [B,K,F], as float64 tensors on n_chi_stack's device."""
    host = lambda v: v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)
    n = n_chi_stack if isinstance(n_chi_stack, torch.Tensor) else torch.as_tensor(np.asarray(n_chi_stack))
    n = n.to(F64)
    dev = n.device
    dom_ins, dom_del = host(dom_ins).astype(float).reshape(-1), host(dom_del).astype(float).reshape(-1)
    dom_w, frag_w = host(dom_weights).astype(float).reshape(-1), host(frag_weights).astype(float)
    ext = host(ext_rates).astype(float)
    K, F = frag_w.shape
    if ext.ndim == 2:
        ext = np.stack([np.diag(ext[k]) for k in range(K)])
    t = host(t_array).astype(float).reshape(-1)
    B = t.shape[0]
    if n.dim() == 2:
        n = n.unsqueeze(0)
    if n.shape[0] != B:
        raise ValueError('n_chi_stack and t_array disagree on the number of pairs')
    L, outs, n_out, dst, src, w = _plan(K, F)
    if n.shape[-1] != 2 + 5 * K * F:
        raise ValueError('n_chi_stack does not match n_dom x n_frag')
    T = torch.as_tensor(_exploded(float(host(main_ins)), float(host(main_del)), t, dom_ins, dom_del, dom_w,
                                  frag_w, ext, L), dtype=F64).to(dev)
    kp = torch.as_tensor(L.kept, device=dev)
    z = torch.as_tensor(L.null, device=dev)
    TKK = T[:, kp][:, :, kp]
    TKZ = T[:, kp][:, :, z]
    TZK = T[:, z][:, :, kp]
    TZZ = T[:, z][:, :, z]
    eye = torch.eye(len(L.null), dtype=F64, device=dev)
    C = torch.linalg.inv(eye - TZZ)
    H = C @ TZK
    Ct = TKZ @ C
    Tred = TKK + Ct @ TZK
    ok = Tred.abs() > 1e-30
    scale = torch.where(ok, n / torch.where(ok, Tred, torch.ones_like(Tred)), torch.zeros_like(Tred))
    CtS = Ct.transpose(1, 2) @ scale
    nf = torch.zeros_like(T)
    nf[:, kp.unsqueeze(1), kp.unsqueeze(0)] = scale * TKK
    nf[:, kp.unsqueeze(1), z.unsqueeze(0)] = TKZ * (scale @ H.transpose(1, 2))
    nf[:, z.unsqueeze(1), kp.unsqueeze(0)] = TZK * CtS
    nf[:, z.unsqueeze(1), z.unsqueeze(0)] = TZZ * (CtS @ H.transpose(1, 2))
    v = torch.cat([nf.reshape(B, -1), nf.sum(dim=2), nf.sum(dim=1)], dim=1)
    flat = torch.zeros(B, n_out, dtype=F64, device=dev)
    flat.index_add_(1, torch.as_tensor(dst, device=dev),
                    v[:, torch.as_tensor(src, device=dev)] * torch.as_tensor(w, device=dev))
    res = {}
    for name, (shape, off) in outs.items():
        res[name] = flat[:, off:off + int(np.prod(shape))].reshape(B, *shape)
    res['dom_M_5x5'] = [res['dom_M_5x5'][:, k] for k in range(K)]
    return res
