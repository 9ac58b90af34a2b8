"""Float64 epilogue of the batched TKF92 E-step: birth-death-immigration
(BDI) sufficient statistics from the expected transition counts.

Restates, batched over pairs in torch float64:
  * the TKF92 chi decomposition (train/tkf92_svi_bw.py:75-122): fragment
    extensions are taken off the M/I/D diagonals, giving the TKF91-style
    resolved counts, the extension count and the body-row total;
  * the log_kappa / log_1mkappa coefficients L, M of the resolved counts
    (train/tkf92_svi_bw.py:160-171);
  * E[B], E[D], E[S] of core/bdi.py:682-780: the WFST log-likelihood with the
    smooth beta / gamma forms (core/bdi.py:101-160), its lambda / mu scores by
    automatic differentiation, the conservation term, and either the general
    formula or, for |1 - kappa| < 1e-10, the L'Hopital limit E[S] = f'(mu).
Negative values from cancellation are clamped at zero as the reference does
(train/tkf92_svi_bw.py:318-320).
"""
from __future__ import annotations

import torch

from . import models as pm

S, M, I, D, E = 0, 1, 2, 3, 4
ES_LHOPITAL_THRESHOLD = 1e-10
F64 = torch.float64


def expm1_ratio(x):
    """(e^x - 1) / x, with its Taylor polynomial for |x| < 1e-5."""
    small = x.abs() < 1e-5
    safe = torch.where(x.abs() < 1e-30, torch.ones_like(x), x)
    return torch.where(small, 1.0 + x / 2.0 + x * x / 6.0 + x * x * x / 24.0, torch.expm1(x) / safe)


def tkf_beta_smooth(lam, mu, t):
    r = expm1_ratio((mu - lam) * t)
    return lam * t * r / (mu * t * r + 1.0)


def tkf_gamma_smooth(lam, mu, t):
    alpha = torch.exp(-mu * t)
    beta = tkf_beta_smooth(lam, mu, t)
    return 1.0 - mu * beta / (lam * torch.clamp(1.0 - alpha, min=1e-30))


def wfst_groups(n):
    """The six WFST coefficient groups of a [..., 5, 5] count matrix (core/bdi.py:353-392)."""
    return {
        'a': n[..., S, M] + n[..., M, M] + n[..., I, M] + n[..., D, M],
        '1a': n[..., S, D] + n[..., M, D] + n[..., I, D] + n[..., D, D],
        'b': n[..., S, I] + n[..., M, I] + n[..., I, I],
        '1b': (n[..., S, M] + n[..., S, D] + n[..., S, E] + n[..., M, M] + n[..., M, D] + n[..., M, E]
               + n[..., I, M] + n[..., I, D] + n[..., I, E]),
        'g': n[..., D, I],
        '1g': n[..., D, M] + n[..., D, D] + n[..., D, E],
    }


def log_p_wfst(lam, mu, t, g):
    """sum_g n_g log(xi_g) with the smooth beta / gamma and a 1e-30 log floor."""
    alpha = torch.exp(-mu * t)
    beta = tkf_beta_smooth(lam, mu, t)
    gamma = tkf_gamma_smooth(lam, mu, t)
    lg = lambda v: torch.log(torch.clamp(v, min=1e-30))
    return (g['a'] * lg(alpha) + g['1a'] * lg(1.0 - alpha) + g['b'] * lg(beta) + g['1b'] * lg(1.0 - beta)
            + g['g'] * lg(gamma) + g['1g'] * lg(1.0 - gamma))


def bdi_stats(n_trans, ins_rate, del_rate, t, T=None):
    """(E_B, E_D, E_S) per pair from resolved TKF91-style counts [B, 5, 5]."""
    n = pm._t(n_trans)
    dev = n.device
    t = pm._t(t, device=dev).reshape(-1)
    T = t if T is None else pm._t(T, device=dev).reshape(-1)
    B = n.shape[0]
    lam0, mu0 = float(ins_rate), float(del_rate)
    g = {k: v.detach() for k, v in wfst_groups(n).items()}
    cons = n[:, :, I].sum(dim=1) - n[:, :, D].sum(dim=1)
    near_equal = abs(1.0 - lam0 / mu0) < ES_LHOPITAL_THRESHOLD
    with torch.enable_grad():
        lam = torch.full((B,), lam0, dtype=F64, device=dev, requires_grad=True)
        mu = torch.full((B,), mu0, dtype=F64, device=dev, requires_grad=True)
        lp = log_p_wfst(lam, mu, t, g).sum()
        d_lam, d_mu = torch.autograd.grad(lp, (lam, mu))
        lam_score = (lam * d_lam).detach()
        mu_score = (mu * d_mu).detach()
        if not near_equal:
            E_S = (cons + mu_score - lam_score - lam0 * T) / (lam0 - mu0)
        else:
            # f(lambda) = cons + mu dlogP/dmu - lambda dlogP/dlambda - lambda T at
            # (lambda, mu); E[S] = f'(mu), the derivative taken at lambda = mu
            lam2 = torch.full((B,), mu0, dtype=F64, device=dev, requires_grad=True)
            mu2 = torch.full((B,), mu0, dtype=F64, device=dev, requires_grad=True)
            lp2 = log_p_wfst(lam2, mu2, t, g).sum()
            d_lam2, d_mu2 = torch.autograd.grad(lp2, (lam2, mu2), create_graph=True)
            f = (cons + mu0 * d_mu2 - lam2 * d_lam2 - lam2 * T).sum()
            E_S = torch.autograd.grad(f, lam2)[0].detach()
    E_B = lam_score + lam0 * E_S + lam0 * T
    E_D = mu_score + mu0 * E_S
    return E_B, E_D, E_S


def tkf92_resolve(n_chi, ins_rate, del_rate, t, ext):
    """TKF92 chi counts [B, 5, 5] -> (resolved counts, ext_count, notext_count)."""
    n = pm._t(n_chi)
    # tau is built on the host from plain scalars; only the result moves to n's device
    tau = pm.tkf92_trans(pm._t(float(ins_rate)), pm._t(float(del_rate)),
                         pm._t(t).reshape(-1).cpu(), float(ext)).to(n.device)
    diag = torch.stack([tau[:, M, M], tau[:, I, I], tau[:, D, D]], dim=-1)
    frac = torch.where(diag > 1e-30, float(ext) / torch.clamp(diag, min=1e-30), torch.zeros_like(diag))
    frac = torch.clamp(frac, 0.0, 1.0)
    loops = torch.stack([n[:, M, M], n[:, I, I], n[:, D, D]], dim=-1)
    ext_count = (frac * loops).sum(dim=-1)
    res = n.clone()
    for a, s in enumerate((M, I, D)):
        res[:, s, s] = (1.0 - frac[:, a]) * loops[:, a]
    notext = res[:, M, :].sum(-1) + res[:, I, :].sum(-1) + res[:, D, :].sum(-1)
    return res, ext_count, notext


def kappa_coefficients(res):
    """L (log_kappa) and M (log_1mkappa) coefficients of resolved counts."""
    L = (res[:, S, M] + res[:, S, D] + res[:, M, M] + res[:, M, D] + res[:, I, M] + res[:, I, D]
         + res[:, D, M] + res[:, D, D])
    Mc = res[:, S, E] + res[:, M, E] + res[:, I, E] + res[:, D, E]
    return L, Mc


def tkf92_bdi_epilogue(n_chi, ins_rate, del_rate, t, ext, T=None):
    """The dict of estep_batch_tkf92 beyond log_p (train/tkf92_svi_bw.py:263-334)."""
    res, ext_count, notext = tkf92_resolve(n_chi, ins_rate, del_rate, t, ext)
    L, Mc = kappa_coefficients(res)
    tt = pm._t(t, device=res.device).reshape(-1)
    E_B, E_D, E_S = bdi_stats(res, ins_rate, del_rate, tt, T)
    zero = torch.zeros_like(E_B)
    return {'B': torch.maximum(E_B, zero), 'D': torch.maximum(E_D, zero), 'S': torch.maximum(E_S, zero),
            'L': L, 'M': Mc, 'T': tt if T is None else pm._t(T, device=res.device).reshape(-1),
            'ext_count': ext_count, 'notext_count': notext, 'n_trans_resolved': res}


def mixfrag_resolve(n_chi, ins_rate, del_rate, t, exts, weights):
    """MixFrag chi counts [B, 3F+2, 3F+2] -> (resolved 5x5 TKF91-type counts
    [B, 5, 5], F_f [B, F] fragment-extension counts, E_f [B, F] fragment-end
    counts), train/mixfrag_svi_bw.py:59-110: the a_f -> a_f self-loop count
    splits into extension, ext_f / (ext_f + (1 - ext_f) tau91[a, a] w_f) of it,
    and a new fragment link; the resolved counts are summed over fragment
    types."""
    n = pm._t(n_chi)
    dev = n.device
    B, ns = n.shape[0], n.shape[1]
    F = (ns - 2) // 3
    exts = pm._t(exts, device=dev).reshape(-1)
    w = pm._t(weights, device=dev).reshape(-1)
    tau91 = pm.tkf91_trans(pm._t(float(ins_rate)), pm._t(float(del_rate)),
                           pm._t(t).reshape(-1).cpu()).to(dev)
    res = n.clone()
    F_f = torch.zeros(B, F, dtype=F64, device=dev)
    E_f = torch.zeros(B, F, dtype=F64, device=dev)
    for k, ty in enumerate((M, I, D)):
        diag = tau91[:, ty, ty]
        for f in range(F):
            a = 1 + k * F + f
            loop = exts[f] + (1.0 - exts[f]) * diag * w[f]
            frac = torch.where(loop > 1e-30, exts[f] / torch.clamp(loop, min=1e-30), torch.zeros_like(loop))
            Faf = torch.clamp(frac, 0.0, 1.0) * n[:, a, a]
            F_f[:, f] += Faf
            E_f[:, f] += n[:, a, :].sum(-1)
            res[:, a, a] -= Faf
    E_f = E_f - F_f
    types = torch.as_tensor(pm.mixfrag_state_types(F), device=dev)
    agg = torch.zeros(5, ns, dtype=F64, device=dev)
    agg[types, torch.arange(ns, device=dev)] = 1.0
    return agg[None] @ res @ agg.T[None], F_f, E_f


def mixfrag_bdi_epilogue(n_chi, ins_rate, del_rate, t, exts, weights):
    """The dict of estep_batch_mixfrag beyond log_p (train/mixfrag_svi_bw.py:194-232):
    B, D, S (BDI statistics of the resolved counts, floored at 0), L, M
    (kappa coefficients), T (= t), F_f, E_f."""
    res5, F_f, E_f = mixfrag_resolve(n_chi, ins_rate, del_rate, t, exts, weights)
    L, Mc = kappa_coefficients(res5)
    tt = pm._t(t, device=res5.device).reshape(-1)
    E_B, E_D, E_S = bdi_stats(res5, ins_rate, del_rate, tt, tt)
    zero = torch.zeros_like(E_B)
    return {'B': torch.maximum(E_B, zero), 'D': torch.maximum(E_D, zero), 'S': torch.maximum(E_S, zero),
            'L': L, 'M': Mc, 'T': tt, 'F_f': F_f, 'E_f': E_f}
