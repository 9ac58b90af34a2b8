"""FP64 restatement of the batched TKF92 E-step epilogue -- TEST INFRASTRUCTURE ONLY.

BDI sufficient statistics from TKF91-style transition counts (core/bdi.py:
101-160 smooth beta / gamma, 353-392 count groups, 682-780 general and
L'Hopital branches) and the TKF92 chi decomposition
(train/tkf92_svi_bw.py:75-122, 160-171).  The lambda / mu derivatives of the
WFST log-likelihood are taken by complex-step differentiation (exact to
rounding); the L'Hopital branch differentiates the complex-step scores by a
central difference.
"""
import numpy as np

from .models import tkf92_trans

S, M, I, D, E = 0, 1, 2, 3, 4


def _expm1_ratio(x):
    x = np.asarray(x, dtype=complex)
    small = np.abs(x) < 1e-5
    safe = np.where(np.abs(x) < 1e-30, 1.0, x)
    return np.where(small, 1.0 + x / 2.0 + x * x / 6.0 + x ** 3 / 24.0, (np.exp(x) - 1.0) / safe)


def _log_p(lam, mu, t, n):
    alpha = np.exp(-mu * t)
    r = _expm1_ratio((mu - lam) * t)
    beta = lam * t * r / (mu * t * r + 1.0)
    Phi = 1.0 - alpha
    Phi = np.where(np.real(Phi) < 1e-30, 1e-30, Phi)
    gamma = 1.0 - mu * beta / (lam * Phi)
    lg = lambda v: np.log(np.where(np.real(v) < 1e-30, 1e-30, v))
    ga = n[S, M] + n[M, M] + n[I, M] + n[D, M]
    g1a = n[S, D] + n[M, D] + n[I, D] + n[D, D]
    gb = n[S, I] + n[M, I] + n[I, I]
    g1b = n[S, M] + n[S, D] + n[S, E] + n[M, M] + n[M, D] + n[M, E] + n[I, M] + n[I, D] + n[I, E]
    gg = n[D, I]
    g1g = n[D, M] + n[D, D] + n[D, E]
    return (ga * lg(alpha) + g1a * lg(1.0 - alpha) + gb * lg(beta) + g1b * lg(1.0 - beta)
            + gg * lg(gamma) + g1g * lg(1.0 - gamma))


def _d_lam(lam, mu, t, n, h=1e-30):
    return float(np.imag(_log_p(lam + 1j * h, mu, t, n)) / h)


def _d_mu(lam, mu, t, n, h=1e-30):
    return float(np.imag(_log_p(lam, mu + 1j * h, t, n)) / h)


def bdi_stats(n, lam, mu, t, T=None):
    """(E_B, E_D, E_S) of one pair (core/bdi.py:682-780)."""
    n = np.asarray(n, float)
    T = t if T is None else T
    lam_score = lam * _d_lam(lam, mu, t, n)
    mu_score = mu * _d_mu(lam, mu, t, n)
    cons = n[:, I].sum() - n[:, D].sum()
    if abs(1.0 - lam / mu) >= 1e-10:
        E_S = (cons + mu_score - lam_score - lam * T) / (lam - mu)
    else:
        f = lambda l: cons + mu * _d_mu(l, mu, t, n) - l * _d_lam(l, mu, t, n) - l * T
        h = 1e-6 * mu
        E_S = (f(mu + h) - f(mu - h)) / (2 * h)
    return lam_score + lam * E_S + lam * T, mu_score + mu * E_S, E_S


def tkf92_epilogue(n_chi, lam, mu, t, ext):
    """dict of one pair: B, D, S, L, M, ext_count, notext_count (train/tkf92_svi_bw.py:131-334)."""
    n = np.asarray(n_chi, float)
    tau = tkf92_trans(lam, mu, t, ext)
    res = n.copy()
    ext_count = 0.0
    for s in (M, I, D):
        frac = ext / tau[s, s] if tau[s, s] > 1e-30 else 0.0
        frac = min(max(frac, 0.0), 1.0)
        ext_count += frac * n[s, s]
        res[s, s] = (1.0 - frac) * n[s, s]
    notext = res[M].sum() + res[I].sum() + res[D].sum()
    L = res[S, M] + res[S, D] + res[M, M] + res[M, D] + res[I, M] + res[I, D] + res[D, M] + res[D, D]
    Mc = res[S, E] + res[M, E] + res[I, E] + res[D, E]
    EB, ED, ES = bdi_stats(res, lam, mu, t)
    return {'B': max(EB, 0.0), 'D': max(ED, 0.0), 'S': max(ES, 0.0), 'L': L, 'M': Mc,
            'ext_count': ext_count, 'notext_count': notext}
