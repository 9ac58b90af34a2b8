"""Generate golden fixtures by running the reference's own pair-HMM modules.

Usage (needs the reference checkout; writes tests/golden/*.npz):

    python tests/golden/make_golden.py <reference>/python

The reference modules (``tkfmixdom/jax/dp/hmm.py``, ``models/mixdom.py``,
``core/params.py``, ``core/bdi.py``, ``core/ctmc.py``,
``train/likelihood.py``, ``train/vjp.py``, ``train/tkf92_svi_bw.py``) are
imported unmodified; JAX itself is replaced by the NumPy stand-in in
``jax_shim.py``.  Inputs are seeded and small enough for the pure-Python
loops of the stand-in.  Every array the fixtures hold is a reference output;
the inputs are stored beside them.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import jax_shim  # noqa: E402


def _load_reference(ref_python):
    jax_shim.install()
    sys.path.insert(0, ref_python)
    from tkfmixdom.jax.dp import hmm
    from tkfmixdom.jax.models import mixdom
    from tkfmixdom.jax.core import params as cparams
    from tkfmixdom.jax.core import ctmc
    from tkfmixdom.jax.train import likelihood, vjp, tkf92_svi_bw
    return dict(hmm=hmm, mixdom=mixdom, params=cparams, ctmc=ctmc,
                likelihood=likelihood, vjp=vjp, svi=tkf92_svi_bw)


def rand_Q_pi(rng, A=20):
    pi = rng.dirichlet(np.ones(A))
    Sx = rng.lognormal(0.0, 1.0, size=(A, A))
    Sx = np.triu(Sx, 1)
    Sx = Sx + Sx.T
    Q = Sx * pi[None, :]
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(axis=1))
    rate = -np.sum(pi * np.diag(Q))
    return Q / rate, pi, Sx / rate


def rand_mixdom2(rng, K, F, C, ext_full):
    cls = [rand_Q_pi(rng) for _ in range(C)]
    p = {
        'main_ins': rng.uniform(0.01, 0.05),
        't': float(np.exp(rng.uniform(np.log(0.05), np.log(2.0)))),
        'dom_ins': rng.uniform(0.01, 0.05, K),
        'dom_weights': rng.dirichlet(np.ones(K)),
        'frag_weights': np.stack([rng.dirichlet(np.ones(F)) for _ in range(K)]),
        'class_pis': np.stack([c[1] for c in cls]),
        'class_S_exch': np.stack([c[2] for c in cls]),
        'classdist': np.stack([[rng.dirichlet(np.ones(C)) for _ in range(F)]
                               for _ in range(K)]),
    }
    p['main_del'] = p['main_ins'] * rng.uniform(1.05, 1.5)
    p['dom_del'] = p['dom_ins'] * rng.uniform(1.05, 1.5, K)
    if ext_full:
        e = rng.uniform(0.05, 0.4, (K, F, F))
        e = e * (rng.uniform(0.3, 0.9, (K, F, 1)) / e.sum(axis=2, keepdims=True))
        p['ext_rates'] = e
    else:
        p['ext_rates'] = rng.uniform(0.3, 0.9, (K, F))
    return p


def seqs(rng, Lx, Ly, A=20, wildcard=False):
    x = rng.integers(0, A, Lx).astype(np.int32)
    y = rng.integers(0, A, Ly).astype(np.int32)
    if wildcard and Lx > 2 and Ly > 2:
        x[1] = 20
        y[2] = 20
    return x, y


def flat(prefix, d):
    return {f'{prefix}{k}': np.asarray(v) for k, v in d.items()}


def main(ref_python):
    R = _load_reference(ref_python)
    hmm, lik, vjp, mixdom = R['hmm'], R['likelihood'], R['vjp'], R['mixdom']
    cp, ctmc = R['params'], R['ctmc']
    rng = np.random.default_rng(20261203)
    out = os.path.join(HERE)

    # ---------------- TKF91 / TKF92 single pair: tables + E-step
    for name, ext, Lx, Ly, wild in (('tkf91', None, 7, 9, False),
                                    ('tkf92', 0.45, 9, 6, False),
                                    ('tkf91_wild', None, 6, 5, True)):
        Q, pi, _ = rand_Q_pi(rng)
        lam = rng.uniform(0.01, 0.05)
        params = {'ins_rate': lam, 'del_rate': lam * rng.uniform(1.05, 1.5),
                  't': float(rng.uniform(0.1, 1.5)), 'Q': Q, 'pi': pi}
        model = 'tkf91'
        if ext is not None:
            params['ext'] = ext
            model = 'tkf92'
        x, y = seqs(rng, Lx, Ly, wildcard=wild)
        sub = ctmc.transition_matrix(Q, params['t'])
        if model == 'tkf91':
            tau = cp.tkf91_trans(params['ins_rate'], params['del_rate'], params['t'])
        else:
            tau = cp.tkf92_trans(params['ins_rate'], params['del_rate'], params['t'], ext)
        st = np.array([0, 1, 2, 3, 4])
        lt = hmm.safe_log(tau)
        ll_f, Ftab = hmm.forward_2d(lt, st, x, y, sub, pi)
        Btab = hmm.backward_2d(lt, st, x, y, sub, pi)
        ll_fb, post, ntr = hmm.forward_backward_2d(lt, st, x, y, sub, pi)
        ll_e, n_e, ss = lik.e_step(model, params, x, y)
        mp = np.array(ss['match_pairs'], dtype=np.float64).reshape(-1, 3)
        np.savez_compressed(
            os.path.join(out, f'{name}.npz'), model=model, x=x, y=y,
            **flat('p_', params), chi=np.asarray(tau), sub=np.asarray(sub),
            ll_forward=ll_f, F=Ftab, B=Btab, ll_fb=ll_fb,
            post=np.asarray(post)[:Lx + 1, :Ly + 1], n_trans=ntr, ll_estep=ll_e,
            n_estep=n_e, match_pairs=mp, **flat('obs_', ss['pi_obs_counts']))
        print('wrote', name, float(ll_fb))

    # ---------------- MixDom2 E-step + VJP emission counts
    cases = (('mixdom2_k3f1c1', 3, 1, 1, False, 11, 8, False),
             ('mixdom2_k2f2c2', 2, 2, 2, True, 8, 10, False),
             ('mixdom2_k1f2c3_wild', 1, 2, 3, False, 7, 6, True))
    for name, K, F, C, ext_full, Lx, Ly, wild in cases:
        p = rand_mixdom2(rng, K, F, C, ext_full)
        x, y = seqs(rng, Lx, Ly, wildcard=wild)
        # inputs enter the reference as JAX arrays (traced under jit/grad), so
        # they get JAX's gather semantics
        p = {k: (jax_shim._wrap(np.asarray(v)) if np.ndim(v) else v) for k, v in p.items()}
        ll, n_trans, ss = lik.e_step_mixdom2(p, x, y)
        chi, _ = mixdom.build_nested_trans(
            p['main_ins'], p['main_del'], p['t'], p['dom_ins'], p['dom_del'],
            p['dom_weights'], p['frag_weights'], p['ext_rates'])
        class_subs = vjp._build_class_subs(p['class_S_exch'], p['class_pis'], p['t'])
        st = mixdom.state_types(K, F)
        log_emit = hmm.pair_hmm_emissions_per_class(
            st, x, y, class_subs, p['class_pis'], p['classdist'], K, F)
        ll_dp, res = vjp._mixdom2_dp_fwd(
            p['main_ins'], p['main_del'], p['t'], p['dom_ins'], p['dom_del'],
            p['dom_weights'], p['frag_weights'], p['ext_rates'],
            class_subs, p['class_pis'], p['classdist'], x, y)
        (n_chi, post, emit, x_pad, y_pad, rLx, rLy) = res[:7]
        mc, Vlin, cdc = vjp._mixdom2_emission_counts(
            class_subs, p['class_pis'], p['classdist'], post, emit,
            x_pad, y_pad, rLx, rLy, K, F)
        ll_fwd_only = vjp._mixdom2_dp(
            p['main_ins'], p['main_del'], p['t'], p['dom_ins'], p['dom_del'],
            p['dom_weights'], p['frag_weights'], p['ext_rates'],
            class_subs, p['class_pis'], p['classdist'], x, y)
        np.savez_compressed(
            os.path.join(out, f'{name}.npz'), K=K, F=F, C=C, x=x, y=y,
            **flat('p_', p), chi=np.asarray(chi), class_subs=np.asarray(class_subs),
            log_emit=np.asarray(log_emit), ll=ll, n_trans=np.asarray(n_trans),
            **flat('ss_', ss), ll_dp=ll_dp, n_chi=np.asarray(n_chi),
            post=np.asarray(post)[:Lx + 1, :Ly + 1], mc_c=np.asarray(mc),
            V_c_linear=np.asarray(Vlin), cd_count=np.asarray(cdc),
            ll_fwd_only=ll_fwd_only)
        print('wrote', name, ll)

    # ---------------- MixDom1 chi from trained parameters + per-domain emissions
    ck = np.load(os.path.join(ref_python, 'params', 'best', 'bw_d3f2_pfam100_20iter.npz'))
    K, F = ck['dom_ins'].shape[0], ck['frag_weights'].shape[1]
    t = 0.7
    chi, _ = mixdom.build_nested_trans(ck['main_ins'], ck['main_del'], t,
                                       ck['dom_ins'], ck['dom_del'], ck['dom_weights'],
                                       ck['frag_weights'], ck['ext_rates'])
    subs = np.stack([ctmc.transition_matrix(ck['dom_Qs'][k], t) for k in range(K)])
    x, y = seqs(rng, 9, 8)
    st = mixdom.state_types(K, F)
    emit = hmm.pair_hmm_emissions_per_domain(st, x, y, subs, ck['dom_pis'], K, F)
    lt = hmm.safe_log(chi)
    ll, post, ntr = hmm.forward_backward_2d(lt, st, x, y, None, None, log_emit_table=emit)
    np.savez_compressed(os.path.join(out, 'mixdom1_d3f2.npz'), K=K, F=F, t=t, x=x, y=y,
                        main_ins=ck['main_ins'], main_del=ck['main_del'],
                        dom_ins=ck['dom_ins'], dom_del=ck['dom_del'],
                        dom_weights=ck['dom_weights'], frag_weights=ck['frag_weights'],
                        ext_rates=ck['ext_rates'], dom_Qs=ck['dom_Qs'],
                        dom_pis=ck['dom_pis'], chi=np.asarray(chi), subs=subs,
                        log_emit=np.asarray(emit), ll=ll,
                        post=np.asarray(post)[:10, :9], n_trans=np.asarray(ntr))
    print('wrote mixdom1_d3f2', ll)

    # ---------------- MixFrag matrix and the builders' small pieces
    lam = 0.02
    mf = cp.mixfrag_trans(lam, lam * 1.3, 0.8, np.array([0.3, 0.7]), np.array([0.6, 0.4]))
    t92 = cp.tkf92_trans(lam, lam * 1.3, 0.8, 0.35)
    t91_lim = cp.tkf91_trans(0.03, 0.03 * (1 + 3e-5), 0.9)
    np.savez_compressed(os.path.join(out, 'builders.npz'), mixfrag=np.asarray(mf),
                        tkf92=np.asarray(t92), tkf91_limit=np.asarray(t91_lim))

    # ---------------- edge cases: empty sequences
    Q, pi, _ = rand_Q_pi(rng)
    params = {'ins_rate': 0.02, 'del_rate': 0.027, 't': 0.6, 'Q': Q, 'pi': pi}
    sub = ctmc.transition_matrix(Q, 0.6)
    tau = cp.tkf91_trans(0.02, 0.027, 0.6)
    lt = hmm.safe_log(tau)
    st = np.array([0, 1, 2, 3, 4])
    edge = {}
    for tag, (Lx, Ly) in {'x0': (0, 4), 'y0': (5, 0), 'xy0': (0, 0), 'x1y1': (1, 1)}.items():
        x, y = seqs(rng, Lx, Ly)
        ll, post, ntr = hmm.forward_backward_2d(lt, st, x, y, sub, pi)
        edge[f'{tag}_x'] = x
        edge[f'{tag}_y'] = y
        edge[f'{tag}_ll'] = ll
        edge[f'{tag}_n'] = np.asarray(ntr)
        edge[f'{tag}_post'] = np.asarray(post)[:Lx + 1, :Ly + 1]
    np.savez_compressed(os.path.join(out, 'edges_tkf91.npz'), Q=Q, pi=pi, chi=tau,
                        sub=sub, **edge)
    print('wrote edges')

    # ---------------- batched (vmap) forward-only over pre-padded pairs
    Q, pi, _ = rand_Q_pi(rng)
    lens = [(5, 7), (8, 6), (7, 7), (3, 8)]
    Lxp = max(hmm._pad_to_bin(a) for a, _ in lens)
    Lyp = max(hmm._pad_to_bin(b) for _, b in lens)
    xs = np.zeros((4, Lxp), np.int32)
    ys = np.zeros((4, Lyp), np.int32)
    for i, (a, b) in enumerate(lens):
        x, y = seqs(rng, a, b)
        xs[i, :a] = x
        ys[i, :b] = y
    ts = np.array([0.3, 0.8, 1.2, 0.5])
    Lxr = np.array([a for a, _ in lens], np.int32)
    Lyr = np.array([b for _, b in lens], np.int32)
    lp = R['svi'].estep_batch_tkf92_forward_only(xs, ys, ts, Lxr, Lyr,
                                                 0.02, 0.028, 0.4, Q, pi)
    np.savez_compressed(os.path.join(out, 'batch_tkf92_fwd.npz'), xs=xs, ys=ys, ts=ts,
                        Lx=Lxr, Ly=Lyr, lam=0.02, mu=0.028, ext=0.4, Q=Q, pi=pi,
                        log_p=np.asarray(lp))
    print('wrote batch', np.asarray(lp))


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden.py <reference checkout>/python')
    main(sys.argv[1])
