"""The reference's custom-VJP cotangents (tests/golden/vjp.npz, made by
tests/golden/make_golden_vjp.py from the reference's own _fwd / _bwd pairs in
train/vjp.py) against central differences of the FP64 oracle's
log-likelihood: the fixtures are checked independently before the GPU tests
compare the CUDA gradients with them."""
import numpy as np
import pytest

from conftest import GOLDEN
from oracle import models as om, dp as odp, estep as oe

G = np.load(GOLDEN + '/vjp.npz')
FD_RTOL = 2e-6


def _ll_tkf(model, q, x, y):
    chi = om.tkf91_trans(q['lam'], q['mu'], q['t']) if model == 'tkf91' else \
        om.tkf92_trans(q['lam'], q['mu'], q['t'], q['ext'])
    sub = om.transition_matrix(q['Q'], q['t'])
    EM, EI, ED = odp.group_tables_tkf(sub, q['pi'])
    st = om.tkf_state_types()
    return odp.forward_table(om.safe_log(chi), st, odp.log_emission_table(st, np.zeros(5, int), x, y, EM, EI, ED))[0]


def _fd(f, q, key, idx):
    """Central differences at h = 1e-3 of the entry and h/2, Richardson-
    extrapolated: the MixDom chi builders (a Gauss-Jordan solve) carry ~1e-13
    relative noise, which steps of 1e-6 would turn into ~3e-5 errors."""
    v = np.array(q[key], dtype=np.float64)
    flat = v.reshape(-1)

    def d(h):
        a, b = flat.copy(), flat.copy()
        a[idx] += h
        b[idx] -= h
        qa, qb = dict(q), dict(q)
        qa[key] = a.reshape(v.shape) if v.ndim else float(a[0])
        qb[key] = b.reshape(v.shape) if v.ndim else float(b[0])
        return (f(qa) - f(qb)) / (2 * h)
    h = 1e-3 * max(abs(flat[idx]), 1e-3)
    return (4.0 * d(h / 2) - d(h)) / 3.0


def _check(f, q, grads, rng, n_per=3):
    for key, g in grads.items():
        g = np.asarray(g, np.float64).reshape(-1)
        for idx in rng.choice(g.size, size=min(n_per, g.size), replace=False):
            want = _fd(f, q, key, idx)
            assert abs(g[idx] - want) <= FD_RTOL * max(abs(want), 1.0), (key, idx, g[idx], want)


@pytest.mark.parametrize('model', ['tkf91', 'tkf92'])
def test_tkf_cotangents_match_oracle_fd(model):
    q = {k: G[f'{model}_{k}'] for k in ('lam', 'mu', 't', 'ext', 'Q', 'pi')}
    q = {k: (float(v) if v.ndim == 0 else v) for k, v in q.items()}
    x, y = G[f'{model}_x'].astype(int), G[f'{model}_y'].astype(int)
    f = lambda qq: _ll_tkf(model, qq, x, y)
    assert abs(f(q) - float(G[f'{model}_ll'])) < 1e-9 * abs(f(q))
    keys = ['lam', 'mu', 't', 'Q', 'pi'] + (['ext'] if model == 'tkf92' else [])
    _check(f, q, {k: G[f'{model}_g_{k}'] for k in keys}, np.random.default_rng(1))


def test_mixdom1_cotangents_match_oracle_fd():
    names = ['main_ins', 'main_del', 't', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates']
    q = {k: G[f'mixdom1_p_{k}'] for k in names}
    q = {k: (float(v) if v.ndim == 0 else v) for k, v in q.items()}
    q['Q'], q['pi'] = G['mixdom1_Q'], G['mixdom1_pi']
    x, y = G['mixdom1_x'].astype(int), G['mixdom1_y'].astype(int)
    K, F = q['frag_weights'].shape

    def f(qq):
        chi = om.build_nested_trans(qq['main_ins'], qq['main_del'], qq['t'], qq['dom_ins'], qq['dom_del'],
                                    qq['dom_weights'], qq['frag_weights'], qq['ext_rates'])
        st = om.mixdom_state_types(K, F)
        EM, EI, ED = odp.group_tables_tkf(om.transition_matrix(qq['Q'], qq['t']), qq['pi'])
        return odp.forward_table(om.safe_log(chi), st,
                                 odp.log_emission_table(st, np.zeros(len(st), int), x, y, EM, EI, ED))[0]
    assert abs(f(q) - float(G['mixdom1_ll'])) < 1e-9 * abs(f(q))
    grads = {k: G[f'mixdom1_ct_{k}'] for k in names if k != 't'}
    grads.update({'t': G['mixdom1_g_t'], 'Q': G['mixdom1_g_Q'], 'pi': G['mixdom1_g_pi']})
    _check(f, q, grads, np.random.default_rng(2))


@pytest.mark.parametrize('name', ['mixdom2_k3f1c1', 'mixdom2_k2f2c2'])
def test_mixdom2_cotangents_match_oracle_fd(name):
    keys = ['main_ins', 'main_del', 't', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates',
            'class_pis', 'class_S_exch', 'classdist']
    q = {k: G[f'{name}_p_{k}'] for k in keys}
    q = {k: (float(v) if v.ndim == 0 else v) for k, v in q.items()}
    x, y = G[f'{name}_x'].astype(int), G[f'{name}_y'].astype(int)

    def f(qq):
        chi, st, groups, EM, EI, ED, _ = oe.mixdom2_model(qq)
        return odp.forward_table(om.safe_log(chi), st, odp.log_emission_table(st, groups, x, y, EM, EI, ED))[0]
    assert abs(f(q) - float(G[f'{name}_ll'])) < 1e-9 * abs(f(q))
    grads = {k: G[f'{name}_ct_{k}'] for k in keys[:8] if k != 't'}
    grads.update({'t': G[f'{name}_g_t'], 'class_S_exch': G[f'{name}_g_class_S_exch'],
                  'class_pis': G[f'{name}_g_class_pis'], 'classdist': G[f'{name}_g_classdist']})
    _check(f, q, grads, np.random.default_rng(3), n_per=4)
