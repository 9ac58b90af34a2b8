"""Golden cotangents of the reference's custom-VJP log-likelihoods.

Usage (needs the reference checkout; writes tests/golden/vjp.npz):

    python tests/golden/make_golden_vjp.py <reference>/python

For each case the reference's own forward / backward pair of its inner
custom VJP (``train/vjp.py``: ``_tkf91_dp_fwd`` / ``_tkf91_dp_bwd`` (143-194),
``_tkf92_dp_fwd`` / ``_tkf92_dp_bwd`` (272-329), ``_mixdom_dp_fwd`` /
``_mixdom_dp_bwd`` (405-458), ``_mixdom2_dp_fwd`` / ``_mixdom2_dp_bwd``
(727-820)) runs unmodified under the NumPy stand-in for JAX
(``jax_shim.py``), with g = 1.  The ``jax.grad`` calls inside those backward
passes (of the closed-form sum n log chi(theta)) are Richardson-extrapolated
central differences in the stand-in.

The outer wrappers (``tkf91_log_prob`` 110, ``tkf92_log_prob`` 253,
``mixdom_log_prob`` 351, ``mixdom2_log_prob`` 628) build the substitution
matrices P = expm(t Q) outside the custom VJP and let JAX differentiate
through ``jax.scipy.linalg.expm`` (Pade, whose VJP is the exact Frechet
adjoint).  That outer chain is applied here exactly: for a cotangent G of P,
W = L(t Q^T, G) (scipy.linalg.expm_frechet, the adjoint of the Frechet
derivative of expm), so dLL/dQ = t W and the substitution side of dLL/dt is
<W, Q>; for MixDom2, Q_c[a,b] = S_c[a,b] pi_c[b] (a != b) with the negative
row sums on the diagonal (``_build_class_Q`` 463-476) carries W on to
class_S_exch and class_pis.  The fixture stores the inner cotangents as the
reference returns them and the total gradients of each public log-likelihood.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import scipy.linalg

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import jax_shim  # noqa: E402
from make_golden import _load_reference, rand_Q_pi, rand_mixdom2, seqs  # noqa: E402


def expm_adjoint(tQ, G):
    """W = L(tQ^T, G): <G, L(tQ, E)> = <W, E> for every direction E."""
    return scipy.linalg.expm_frechet(np.asarray(tQ).T, np.asarray(G), compute_expm=False)


def class_Q_chain(S, pi, t, W):
    """dLL/dS, dLL/dpi (through Q only) and the t term for one class, given
    W = dLL/d(tQ) and Q[a,b] = S[a,b] pi[b] (a != b), Q[a,a] = -sum_b Q[a,b]."""
    A = pi.size
    tW = t * W
    D = tW - np.diag(tW)[:, None]          # dLL/dQ[a,b] - dLL/dQ[a,a]
    off = ~np.eye(A, dtype=bool)
    gS = np.where(off, D * pi[None, :], 0.0)
    gpi = np.where(off, D * S, 0.0).sum(axis=0)
    return gS, gpi


def main(ref_python):
    R = _load_reference(ref_python)
    vjp, ctmc, cp, mixdom = R['vjp'], R['ctmc'], R['params'], R['mixdom']
    rng = np.random.default_rng(20261204)
    out = {}

    # ---------------- TKF91 / TKF92 (tkf91_log_prob, tkf92_log_prob)
    for name, ext in (('tkf91', None), ('tkf92', 0.4)):
        Q, pi, _ = rand_Q_pi(rng)
        lam = float(rng.uniform(0.01, 0.05))
        mu = lam * float(rng.uniform(1.05, 1.5))
        t = float(rng.uniform(0.2, 1.5))
        x, y = seqs(rng, 9, 8)
        sub = np.asarray(ctmc.transition_matrix(Q, t))
        if ext is None:
            ll, res = vjp._tkf91_dp_fwd(lam, mu, t, sub, pi, x, y)
            d_lam, d_mu, d_t, d_sub, d_pi, _, _ = vjp._tkf91_dp_bwd(res, 1.0)
            d_ext = 0.0
        else:
            ll, res = vjp._tkf92_dp_fwd(lam, mu, t, ext, sub, pi, x, y)
            d_lam, d_mu, d_t, d_ext, d_sub, d_pi, _, _ = vjp._tkf92_dp_bwd(res, 1.0)
        W = expm_adjoint(t * Q, d_sub)
        out.update({f'{name}_{k}': np.asarray(v, np.float64) for k, v in dict(
            x=x, y=y, Q=Q, pi=pi, lam=lam, mu=mu, t=t, ext=ext if ext is not None else 0.0, ll=ll,
            ct_lam=d_lam, ct_mu=d_mu, ct_t_chi=d_t, ct_ext=d_ext, ct_sub=d_sub, ct_pi=d_pi,
            g_lam=d_lam, g_mu=d_mu, g_t=float(d_t) + float((W * Q).sum()), g_ext=d_ext, g_Q=t * W,
            g_pi=d_pi).items()})
        print('wrote', name, float(ll))

    # ---------------- MixDom1 (mixdom_log_prob)
    K, F = 2, 1
    p = rand_mixdom2(rng, K, F, 1, False)
    Q, pi, _ = rand_Q_pi(rng)
    x, y = seqs(rng, 8, 9)
    t = float(p['t'])
    sub = np.asarray(ctmc.transition_matrix(Q, t))
    args = [p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'], p['dom_weights'], p['frag_weights'],
            p['ext_rates']]
    args = [jax_shim._wrap(np.asarray(a)) if np.ndim(a) else a for a in args]
    ll, res = vjp._mixdom_dp_fwd(*args, sub, pi, x, y)
    g = vjp._mixdom_dp_bwd(res, 1.0)
    W = expm_adjoint(t * Q, g[8])
    names = ['main_ins', 'main_del', 't', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates']
    out.update({f'mixdom1_p_{k}': np.asarray(a, np.float64) for k, a in zip(names, args)})
    out.update({f'mixdom1_ct_{k}': np.asarray(v, np.float64) for k, v in zip(names, g[:8])})
    out.update({'mixdom1_x': x, 'mixdom1_y': y, 'mixdom1_Q': Q, 'mixdom1_pi': pi, 'mixdom1_ll': ll,
                'mixdom1_ct_sub': np.asarray(g[8]), 'mixdom1_ct_pi': np.asarray(g[9]),
                'mixdom1_g_t': float(g[2]) + float((W * Q).sum()), 'mixdom1_g_Q': t * W,
                'mixdom1_g_pi': np.asarray(g[9])})
    print('wrote mixdom1', float(ll))

    # ---------------- MixDom2 (mixdom2_log_prob)
    for name, K, F, C, ext_full, Lx, Ly in (('mixdom2_k3f1c1', 3, 1, 1, False, 9, 8),
                                            ('mixdom2_k2f2c2', 2, 2, 2, True, 8, 7)):
        p = rand_mixdom2(rng, K, F, C, ext_full)
        p = {k: (jax_shim._wrap(np.asarray(v)) if np.ndim(v) else v) for k, v in p.items()}
        x, y = seqs(rng, Lx, Ly)
        t = float(p['t'])
        csubs = np.asarray(vjp._build_class_subs(p['class_S_exch'], p['class_pis'], t))
        args = [p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'], p['dom_weights'], p['frag_weights'],
                p['ext_rates']]
        ll, res = vjp._mixdom2_dp_fwd(*args, csubs, p['class_pis'], p['classdist'], x, y)
        g = vjp._mixdom2_dp_bwd(res, 1.0)
        g_cs, g_pi_lin, g_cd = (np.asarray(v) for v in g[8:11])
        gS = np.zeros((C, 20, 20))
        gpi = np.array(g_pi_lin, dtype=np.float64)
        gt = float(g[2])
        for c in range(C):
            Qc = np.asarray(vjp._build_class_Q(p['class_S_exch'][c], p['class_pis'][c]))
            Wc = expm_adjoint(t * Qc, g_cs[c])
            gt += float((Wc * Qc).sum())
            sc, pc = class_Q_chain(np.asarray(p['class_S_exch'][c]), np.asarray(p['class_pis'][c]), t, Wc)
            gS[c] = sc
            gpi[c] += pc
        out.update({f'{name}_p_{k}': np.asarray(v, np.float64) for k, v in p.items()})
        out.update({f'{name}_ct_{k}': np.asarray(v, np.float64) for k, v in zip(names, g[:8])})
        out.update({f'{name}_x': x, f'{name}_y': y, f'{name}_ll': ll, f'{name}_ct_class_subs': g_cs,
                    f'{name}_ct_class_pis_linear': g_pi_lin, f'{name}_ct_classdist': g_cd,
                    f'{name}_g_t': gt, f'{name}_g_class_S_exch': gS, f'{name}_g_class_pis': gpi,
                    f'{name}_g_classdist': g_cd, f'{name}_K': K, f'{name}_F': F, f'{name}_C': C})
        print('wrote', name, float(ll))
    np.savez_compressed(os.path.join(HERE, 'vjp.npz'), **out)


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden_vjp.py <reference checkout>/python')
    main(sys.argv[1])
