"""FP64 oracle: pair-HMM parameter builders (TEST INFRASTRUCTURE ONLY).

This module is part of the CPU oracle used by the test-suite, by
``__graft_entry__.smoke()`` and by ``bench.py``'s CPU-baseline leg to check
the CUDA path.  The product (``pairhmm`` package, CUDA library) never
imports it.

Every function restates, in plain NumPy float64, an algorithm of the
reference (evoldoers/tkf-mixdom, ``python/tkfmixdom/jax/...``); the citation
is given per function.  Parity of this restatement against the reference's
own code is pinned by ``tests/golden`` fixtures that were produced by running
the unmodified reference modules under a NumPy stand-in for the JAX API
(``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg

# State-type codes (core/params.py:21).
S, M, I, D, E = 0, 1, 2, 3, 4
NEG_INF = -1e30                       # dp/hmm.py:108
EQUAL_RATE_THRESHOLD = 1e-4           # core/bdi.py:15


def safe_log(x):
    """log with structural zeros mapped to NEG_INF (dp/hmm.py:111-123)."""
    x = np.asarray(x, dtype=np.float64)
    out = np.full(x.shape, NEG_INF)
    pos = x > 0
    out[pos] = np.log(x[pos])
    return out


# ---------------------------------------------------------------- BDI
def tkf_alpha(mu, t):
    """alpha = exp(-mu t) (core/bdi.py:40-42)."""
    return np.exp(-mu * t)


def tkf_beta(lam, mu, t):
    """beta with the L'Hopital branch at lambda ~ mu (core/bdi.py:45-66)."""
    s = mu * t
    eta = np.exp(-lam * t)
    alpha = np.exp(-s)
    numer = lam * (eta - alpha)
    denom = mu * eta - lam * alpha
    if abs(denom) < 1e-30:
        general = 0.0
    else:
        general = numer / denom
    limit = s / (1.0 + s)
    kappa = lam / mu
    return limit if abs(1.0 - kappa) < EQUAL_RATE_THRESHOLD else general


def tkf_gamma(lam, mu, t):
    """gamma with the L'Hopital branch (core/bdi.py:69-91)."""
    s = mu * t
    alpha = tkf_alpha(mu, t)
    beta = tkf_beta(lam, mu, t)
    Phi = 1.0 - alpha
    if abs(Phi) < 1e-30:
        general = 0.0
    else:
        general = 1.0 - mu * beta / (lam * max(Phi, 1e-30))
    phi = 1.0 - s / 2.0 if s < 1e-10 else Phi / max(s, 1e-30)
    limit = 1.0 - 1.0 / ((1.0 + s) * phi)
    kappa = lam / mu
    return limit if abs(1.0 - kappa) < EQUAL_RATE_THRESHOLD else general


def tkf_kappa(lam, mu):
    """kappa = lambda / mu (core/bdi.py:94-96)."""
    return lam / mu


def tkf91_trans(lam, mu, t):
    """5x5 TKF91 pair-HMM matrix, order S,M,I,D,E (core/params.py:29-54)."""
    a = tkf_alpha(mu, t)
    b = tkf_beta(lam, mu, t)
    g = tkf_gamma(lam, mu, t)
    k = tkf_kappa(lam, mu)
    tau = np.zeros((5, 5))
    for src in (S, M, I):
        tau[src, M] = (1 - b) * k * a
        tau[src, I] = b
        tau[src, D] = (1 - b) * k * (1 - a)
        tau[src, E] = (1 - b) * (1 - k)
    tau[D, M] = (1 - g) * k * a
    tau[D, I] = g
    tau[D, D] = (1 - g) * k * (1 - a)
    tau[D, E] = (1 - g) * (1 - k)
    return tau


def tkf91_trans_cond(lam, mu, t):
    """TKF91 matrix conditioned on the ancestor length (core/params.py:57-90):
    kappa removed from the M/D entries and (1 - kappa) from the E entries."""
    a = tkf_alpha(mu, t)
    b = tkf_beta(lam, mu, t)
    g = tkf_gamma(lam, mu, t)
    tau = np.zeros((5, 5))
    for src in (S, M, I):
        tau[src, M] = (1 - b) * a
        tau[src, I] = b
        tau[src, D] = (1 - b) * (1 - a)
        tau[src, E] = 1 - b
    tau[D, M] = (1 - g) * a
    tau[D, I] = g
    tau[D, D] = (1 - g) * (1 - a)
    tau[D, E] = 1 - g
    return tau


def tkf92_trans(lam, mu, t, ext):
    """5x5 TKF92 matrix: fragment self-loops on M,I,D (core/params.py:92-124)."""
    t91 = tkf91_trans(lam, mu, t)
    tau = np.zeros((5, 5))
    tau[S] = t91[S]
    for src in (M, I, D):
        tau[src] = (1 - ext) * t91[src]
        tau[src, src] = ext + (1 - ext) * t91[src, src]
    return tau


def mixfrag_trans(lam, mu, t, exts, weights):
    """(3F+2)-state MixFrag matrix, order S, M_f, I_f, D_f, E (core/params.py:136-179)."""
    exts = np.asarray(exts, dtype=np.float64)
    weights = np.asarray(weights, dtype=np.float64)
    t91 = tkf91_trans(lam, mu, t)
    F = exts.shape[0]
    Sx, M0, I0, D0, Ex = 0, 1, 1 + F, 1 + 2 * F, 3 * F + 1
    n = 3 * F + 2
    blocks = ((M0, M), (I0, I), (D0, D))
    tau = np.zeros((n, n))
    for db, dty in blocks:
        for gg in range(F):
            tau[Sx, db + gg] = weights[gg] * t91[S, dty]
    tau[Sx, Ex] = t91[S, E]
    for sb, sty in blocks:
        for f in range(F):
            src = sb + f
            for db, dty in blocks:
                for gg in range(F):
                    val = (1.0 - exts[f]) * weights[gg] * t91[sty, dty]
                    if sty == dty and f == gg:
                        val += exts[f]
                    tau[src, db + gg] = val
            tau[src, Ex] = (1.0 - exts[f]) * t91[sty, E]
    return tau


def tkf_state_types():
    return np.array([S, M, I, D, E], dtype=np.int32)


def mixfrag_state_types(F):
    return np.array([S] + [M] * F + [I] * F + [D] * F + [E], dtype=np.int32)


# ---------------------------------------------------------------- MixDom
_UV_EMIT = np.array([M, I, D, I, D])          # models/mixdom.py:66
_UV_U = np.array([M, M, M, I, D])             # models/mixdom.py:244
_UV_X = np.array([M, I, D, I, D])             # models/mixdom.py:246
_IS_M_TYPE = np.array([True, True, True, False, False])
_MID = np.array([M, I, D])


def mixdom_n_states(K, F):
    return 2 + 5 * K * F                      # models/mixdom.py:60-62


def mixdom_state_types(K, F):
    """0=S, 1=E, body 2 + d*5F + uv*F + f with uv->type MM:M MI:I MD:D II:I DD:D
    (models/mixdom.py:52-77)."""
    body = np.tile(np.repeat(_UV_EMIT, F), K)
    return np.concatenate([[S, E], body]).astype(np.int32)


def mixdom_state_groups(K, F):
    """Emission group (d*F+f) of each state; -1 for SS/EE.

    The (d, f) decoding is the one used by the MixDom2 per-class emission
    builder (dp/hmm.py:719-729)."""
    N = mixdom_n_states(K, F)
    g = -np.ones(N, dtype=np.int32)
    body = np.arange(N - 2)
    d = body // (5 * F)
    f = (body % (5 * F)) % F
    g[2:] = d * F + f
    return g


def effective_trans_per_type(main_ins, main_del, t, dom_ins, dom_del, dom_w):
    """Exit-type-resolved 5x5 effective transitions with null states
    eliminated (models/mixdom.py:104-214)."""
    dom_ins = np.asarray(dom_ins, float)
    dom_del = np.asarray(dom_del, float)
    dom_w = np.asarray(dom_w, float)
    K = dom_ins.shape[0]
    tau = tkf91_trans(main_ins, main_del, t)
    kappas = dom_ins / dom_del
    betas = np.array([tkf_beta(dom_ins[k], dom_del[k], t) for k in range(K)])
    z_t = (1.0 - kappas) * (1.0 - betas)
    z_0 = 1.0 - kappas
    tau_rows = np.stack([tau[S], tau[M], tau[I], tau[D], np.zeros(5)])
    tau_MID = tau_rows[:, _MID]                               # (5, 3)
    w_rep = np.repeat(dom_w, 3)
    T_Nnull = np.tile(tau_MID, (1, K)) * w_rep[None, :]       # (5, 3K)
    nonnull = np.stack([1.0 - z_t, kappas, kappas], axis=1)  # (K, 3)
    null_prob = np.stack([z_t, z_0, z_0], axis=1)
    tau_E = np.stack([np.full(K, tau[M, E]), np.full(K, tau[M, E]),
                      np.full(K, tau[D, E])], axis=1)
    T_nullN = np.zeros((3 * K, 5))
    for e in range(3):
        rows = np.arange(K) * 3 + e
        T_nullN[rows, _MID[e]] = nonnull[:, e]
        T_nullN[rows, E] = null_prob[:, e] * tau_E[:, e]
    tau_null_MID = np.stack([tau[M], tau[M], tau[D]])[:, _MID]   # (3, 3)
    z_flat = null_prob.reshape(3 * K)
    ie = np.arange(3 * K) % 3
    jk = np.arange(3 * K) // 3
    je = np.arange(3 * K) % 3
    T_nullnull = (z_flat[:, None] * dom_w[jk[None, :]]
                  * tau_null_MID[ie[:, None], je[None, :]])
    closure = np.linalg.inv(np.eye(3 * K) - T_nullnull)
    closure_3d = closure.reshape(3 * K, K, 3)
    T_nullN_3d = T_nullN.reshape(K, 3, 5)
    closure_exit = np.einsum('ike,kev->kiv', closure_3d, T_nullN_3d)
    T_exit_k = np.einsum('ui,kiv->kuv', T_Nnull, closure_exit)
    T_NN = np.zeros((5, 5))
    T_NN[:, E] = tau_rows[:, E]
    return T_exit_k, T_NN + T_exit_k.sum(axis=0)


def build_nested_trans(main_ins, main_del, t, dom_ins, dom_del, dom_w,
                       frag_w, ext_rates):
    """Collapsed MixDom chi, N = 2 + 5KF, linear space
    (models/mixdom.py:252-423).  ext_rates is (K,F) (diagonal, MixDom1) or
    (K,F,F) (MixDom2)."""
    dom_ins = np.asarray(dom_ins, float)
    dom_del = np.asarray(dom_del, float)
    dom_w = np.asarray(dom_w, float)
    frag_w = np.asarray(frag_w, float)
    ext = np.asarray(ext_rates, float)
    if ext.ndim == 2:
        ext = np.stack([np.diag(r) for r in ext])
    K = dom_ins.shape[0]
    F = frag_w.shape[1]
    nb = K * 5 * F
    N = 2 + nb
    T_exit_k, T = effective_trans_per_type(main_ins, main_del, t,
                                           dom_ins, dom_del, dom_w)
    tau_all = np.stack([tkf91_trans(dom_ins[k], dom_del[k], t) for k in range(K)])
    kappas = dom_ins / dom_del
    beta_d = np.maximum(1.0 - tau_all[:, S, E], 1e-30)
    entry_M = tau_all[:, S, :][:, _UV_X] / beta_d[:, None]
    entry = np.where(_IS_M_TYPE[None, :], entry_M, np.ones((K, 5)))
    exit_M = tau_all[:, :, E][:, _UV_X]
    exit_ID = (1.0 - kappas)[:, None] * np.ones(5)[None, :]
    exit_inner = np.where(_IS_M_TYPE[None, :], exit_M, exit_ID)
    notext = 1.0 - ext.sum(axis=-1)                          # (K, F)
    exit_full = notext[:, None, :] * exit_inner[:, :, None]  # (K, 5, F)

    exit_flat = exit_full.reshape(nb)
    dest_flat = (frag_w[:, None, :] * entry[:, :, None]).reshape(nb)
    T_kc = T_exit_k[:, _UV_U][:, :, _UV_U]                   # (K, 5, 5)
    bs = 5 * F
    d_idx = np.arange(nb) // bs
    suv = np.tile(np.repeat(np.arange(5), F), K)
    T_exp = T_kc[d_idx[None, :], suv[:, None], suv[None, :]]
    chi_inter = exit_flat[:, None] * T_exp * dest_flat[None, :]

    tau_MID_all = tau_all[:, _MID][:, :, _MID]
    nonext_M = np.einsum('df,dxy,dg->dxfyg', notext, tau_MID_all,
                         frag_w).reshape(K, 3 * F, 3 * F)
    ext_M = np.stack([scipy.linalg.block_diag(e, e, e) for e in ext])
    intra_M = nonext_M + ext_M
    nonext_I = notext[:, :, None] * kappas[:, None, None] * frag_w[:, None, :]
    intra_I = nonext_I + ext
    intra_D = nonext_I + ext
    blocks = np.stack([scipy.linalg.block_diag(intra_M[k], intra_I[k], intra_D[k])
                       for k in range(K)])
    loc = np.arange(nb) % bs
    same = d_idx[:, None] == d_idx[None, :]
    chi_intra = blocks[d_idx[:, None], loc[:, None], loc[None, :]] * same
    chi_body = chi_inter + chi_intra

    ss_T = T_exit_k[:, S, :][:, _UV_U]
    ss_body = (ss_T[:, :, None] * frag_w[:, None, :] * entry[:, :, None]).reshape(nb)
    ee_body = (exit_full * T[_UV_U, E][None, :, None]).reshape(nb)

    chi = np.zeros((N, N))
    chi[0, 1] = T[S, E]
    chi[0, 2:] = ss_body
    chi[2:, 1] = ee_body
    chi[2:, 2:] = chi_body
    return chi


# ---------------------------------------------------------------- CTMC
def build_class_Q(S_exch, pi):
    """Q[a,b] = S[a,b] pi[b] off-diagonal, rows sum to zero, no rate
    normalisation (train/vjp.py:463-476)."""
    Q = np.asarray(S_exch, float) * np.asarray(pi, float)[None, :]
    Q = Q - np.diag(np.diag(Q))
    return Q - np.diag(Q.sum(axis=1))


def transition_matrix(Q, t):
    """P(t) = expm(t Q) by Pade scaling and squaring (core/ctmc.py:31-60)."""
    return scipy.linalg.expm(float(t) * np.asarray(Q, float))


def build_class_subs(class_S_exch, class_pis, t):
    """Per-class P_c(t) (train/vjp.py:478-510)."""
    return np.stack([transition_matrix(build_class_Q(Sx, p), t)
                     for Sx, p in zip(class_S_exch, class_pis)])


def holmes_rubin_integrals(Q, pi, t):
    """Holmes-Rubin I[a,b,i,j] and M(t) by the symmetrised eigendecomposition
    (core/ctmc.py:173-230)."""
    Q = np.asarray(Q, float)
    pi = np.asarray(pi, float)
    sp = np.sqrt(pi)
    Sm = Q * (sp[:, None] / sp[None, :])
    Sm = (Sm + Sm.T) / 2
    lam, V = np.linalg.eigh(Sm)
    ex = np.exp(lam * t)
    diff = lam[:, None] - lam[None, :]
    deg = np.abs(diff) < 1e-10
    safe = np.where(deg, 1.0, diff)
    J = np.where(deg, t * ex[:, None], (ex[:, None] - ex[None, :]) / safe)
    VV = V[:, None, :] * V[None, :, :]
    I_sym = np.einsum('aik,kl,jbl->aibj', VV, J, VV)
    pf = np.sqrt((pi[None, None, :, None] * pi[None, :, None, None])
                 / (pi[:, None, None, None] * pi[None, None, None, :] + 1e-30))
    I = I_sym.transpose(0, 2, 1, 3) * pf.transpose(0, 2, 1, 3)
    Msym = (V * ex[None, :]) @ V.T
    Mt = Msym * (sp[None, :] / sp[:, None])
    return I, Mt


def holmes_rubin_weighted_stats(Q, pi, t, mc):
    """W[i], U[i,j] = sum_ab mc[a,b] (dwell, jumps) (core/ctmc.py:285-326)."""
    I, Mt = holmes_rubin_integrals(Q, pi, t)
    Ms = np.where(np.abs(Mt) < 1e-30, 1.0, Mt)
    ratio = np.asarray(mc, float) / Ms
    W = np.einsum('ab,abii->i', ratio, I)
    U = np.asarray(Q, float) * np.einsum('ab,abij->ij', ratio, I)
    return W, U - np.diag(np.diag(U))
