"""Gradients of the differentiable log-likelihoods (torch.autograd.Function
over the CUDA E-step, score identity) against central finite differences of
the float64 oracle: MixDom1 (train/vjp.py:351-458), TKF91 conditioned on the
ancestor length (train/vjp.py:198-249) and MixDom2 with n_dom=4, n_frag=2,
n_classes=2 (42 states, train/vjp.py:627-820)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
LL_RTOL = 1e-6
GRAD_RTOL = 2e-4


def _fd_check(names, p, tens, oracle_ll, n_per=2, seed=0):
    rng = np.random.default_rng(seed)
    for k in names:
        v = np.asarray(p[k], float)
        flat = v.reshape(-1)
        for idx in rng.choice(flat.size, size=min(n_per, flat.size), replace=False):
            h = 1e-6 * max(abs(flat[idx]), 1e-3)
            pp, pm_ = dict(p), dict(p)
            a = flat.copy(); a[idx] += h
            b = flat.copy(); b[idx] -= h
            pp[k] = a.reshape(v.shape) if v.ndim else float(a[0])
            pm_[k] = b.reshape(v.shape) if v.ndim else float(b[0])
            fd = (oracle_ll(pp) - oracle_ll(pm_)) / (2 * h)
            got = tens[k].grad.numpy().reshape(-1)[idx]
            assert abs(got - fd) <= GRAD_RTOL * max(abs(fd), 1.0), (k, idx, got, fd)


def _seqs(rng, lx, ly):
    return rng.integers(0, 20, lx), rng.integers(0, 20, ly)


def test_mixdom1_log_prob_and_gradient(cuda_lib):
    from pairhmm import api, synth
    from oracle import models as om, dp as odp
    rng = np.random.default_rng(3)
    K, F = 2, 1
    p = synth.mixdom2_params(rng, K, F, 1)
    Q, pi, _ = synth.rand_Q_pi(rng)
    p = {k: p[k] for k in ('main_ins', 'main_del', 't', 'dom_ins', 'dom_del', 'dom_weights',
                           'frag_weights', 'ext_rates')}
    p['Q'], p['pi'] = Q, pi
    x, y = _seqs(rng, 23, 19)
    names = list(p)
    tens = {k: torch.tensor(np.asarray(p[k], float), dtype=torch.float64, requires_grad=True) for k in names}
    ll = api.mixdom_log_prob(*[tens[k] for k in names], x, y)
    ll.backward()

    def oracle_ll(q):
        chi = om.build_nested_trans(q['main_ins'], q['main_del'], q['t'], q['dom_ins'], q['dom_del'],
                                    q['dom_weights'], q['frag_weights'], q['ext_rates'])
        st = om.mixdom_state_types(K, F)
        sub = om.transition_matrix(q['Q'], q['t'])
        EM, EI, ED = odp.group_tables_tkf(sub, q['pi'])
        emit = odp.log_emission_table(st, np.zeros(len(st), int), x, y, EM, EI, ED)
        return odp.forward_table(om.safe_log(chi), st, emit)[0]
    want = oracle_ll(p)
    assert abs(float(ll) - want) <= LL_RTOL * abs(want)
    _fd_check(names, p, tens, oracle_ll)


def test_tkf91_conditional_log_prob_and_gradient(cuda_lib):
    from pairhmm import api, synth
    from oracle import models as om, dp as odp
    rng = np.random.default_rng(5)
    p = synth.tkf_params(rng)
    x, y = _seqs(rng, 31, 27)
    names = ['ins_rate', 'del_rate', 't', 'Q', 'pi']
    tens = {k: torch.tensor(np.asarray(p[k], float), dtype=torch.float64, requires_grad=True) for k in names}
    ll = api.tkf91_log_prob_cond(*[tens[k] for k in names], x, y)
    ll.backward()

    def oracle_ll(q):
        chi = om.tkf91_trans_cond(q['ins_rate'], q['del_rate'], q['t'])
        sub = om.transition_matrix(q['Q'], q['t'])
        EM, EI, ED = odp.group_tables_tkf(sub, q['pi'])
        st = om.tkf_state_types()
        emit = odp.log_emission_table(st, np.zeros(5, int), x, y, EM, EI, ED)
        return odp.forward_table(om.safe_log(chi), st, emit)[0]
    want = oracle_ll(p)
    assert abs(float(ll) - want) <= LL_RTOL * abs(want)
    _fd_check(names, p, tens, oracle_ll)


def test_mixdom2_42_states_batched_gradient(cuda_lib):
    """n_dom=4, n_frag=2, n_classes=2: d(sum_p LL_p)/d(theta) for a batch of
    pairs with per-pair t, against central FD of the oracle's summed LL."""
    from pairhmm import api, synth
    from oracle import models as om, dp as odp, estep as oe
    rng = np.random.default_rng(9)
    p = synth.mixdom2_params(rng, 4, 2, 2)
    pairs = [_seqs(rng, int(rng.integers(20, 45)), int(rng.integers(20, 45))) for _ in range(3)]
    ts = np.exp(rng.uniform(np.log(0.1), np.log(1.5), len(pairs)))
    names = ['main_ins', 'main_del', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates',
             'class_pis', 'class_S_exch', 'classdist']
    tens = {k: torch.tensor(np.asarray(p[k], float), dtype=torch.float64, requires_grad=True) for k in names}
    tt = torch.tensor(ts, dtype=torch.float64, requires_grad=True)
    ll = api.mixdom2_log_prob(tens['main_ins'], tens['main_del'], tt, tens['dom_ins'], tens['dom_del'],
                              tens['dom_weights'], tens['frag_weights'], tens['ext_rates'],
                              tens['class_pis'], tens['class_S_exch'], tens['classdist'],
                              [a for a, _ in pairs], [b for _, b in pairs])
    ll.sum().backward()

    def oracle_sum(q, tv=ts):
        tot = 0.0
        for (x, y), t in zip(pairs, tv):
            chi, st, groups, EM, EI, ED, _ = oe.mixdom2_model(dict(q, t=float(t)))
            emit = odp.log_emission_table(st, groups, x, y, EM, EI, ED)
            tot += odp.forward_table(om.safe_log(chi), st, emit)[0]
        return tot
    want = oracle_sum(p)
    assert abs(float(ll.sum()) - want) <= LL_RTOL * abs(want)
    _fd_check(names, p, tens, oracle_sum, n_per=1)
    # per-pair t
    for i in range(len(ts)):
        h = 1e-6 * ts[i]
        a, b = ts.copy(), ts.copy()
        a[i] += h
        b[i] -= h
        fd = (oracle_sum(p, a) - oracle_sum(p, b)) / (2 * h)
        assert abs(float(tt.grad[i]) - fd) <= GRAD_RTOL * max(abs(fd), 1.0), (i, float(tt.grad[i]), fd)
