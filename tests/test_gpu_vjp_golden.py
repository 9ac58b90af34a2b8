"""Gradients of the differentiable log-likelihoods against the reference's own
custom-VJP cotangents (tests/golden/vjp.npz: the reference's _fwd / _bwd pairs
of train/vjp.py with g = 1, chained through expm as JAX does; pinned against
central differences of the FP64 oracle in tests/test_vjp_golden_cpu.py).

tkf91_log_prob (vjp.py:110), tkf92_log_prob (253), mixdom_log_prob (351) and
mixdom2_log_prob (628) run here on the CUDA E-step with the score-identity
adjoint; every gradient entry must equal the reference's within 2e-5 of
max(|g|, 1), and the log-likelihoods within 1e-6 relative."""
import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
LL_RTOL = 1e-6
GRAD_RTOL = 2e-5
G = np.load(GOLDEN + '/vjp.npz')


def _t(v):
    return torch.tensor(np.asarray(v, np.float64), dtype=torch.float64, requires_grad=True)


def _close(got, want, what):
    got = got.detach().cpu().numpy().reshape(-1)
    want = np.asarray(want, np.float64).reshape(-1)
    err = np.abs(got - want) / np.maximum(np.abs(want), 1.0)
    assert err.max() <= GRAD_RTOL, (what, int(err.argmax()), got[err.argmax()], want[err.argmax()], err.max())


@pytest.mark.parametrize('model', ['tkf91', 'tkf92'])
def test_tkf_log_prob_gradients(cuda_lib, model):
    from pairhmm import api
    x, y = G[f'{model}_x'].astype(np.int64), G[f'{model}_y'].astype(np.int64)
    v = {k: _t(G[f'{model}_{k}']) for k in ('lam', 'mu', 't', 'ext', 'Q', 'pi')}
    if model == 'tkf91':
        ll = api.tkf91_log_prob(v['lam'], v['mu'], v['t'], v['Q'], v['pi'], x, y)
    else:
        ll = api.tkf92_log_prob(v['lam'], v['mu'], v['t'], v['ext'], v['Q'], v['pi'], x, y)
    ll.backward()
    want_ll = float(G[f'{model}_ll'])
    assert abs(float(ll.detach()) - want_ll) <= LL_RTOL * abs(want_ll)
    keys = ['lam', 'mu', 't', 'Q', 'pi'] + (['ext'] if model == 'tkf92' else [])
    for k in keys:
        _close(v[k].grad, G[f'{model}_g_{k}'], (model, k))


def test_mixdom1_log_prob_gradients(cuda_lib):
    from pairhmm import api
    names = ['main_ins', 'main_del', 't', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates']
    v = {k: _t(G[f'mixdom1_p_{k}']) for k in names}
    v['Q'], v['pi'] = _t(G['mixdom1_Q']), _t(G['mixdom1_pi'])
    x, y = G['mixdom1_x'].astype(np.int64), G['mixdom1_y'].astype(np.int64)
    ll = api.mixdom_log_prob(*[v[k] for k in names], v['Q'], v['pi'], x, y)
    ll.backward()
    assert abs(float(ll.detach()) - float(G['mixdom1_ll'])) <= LL_RTOL * abs(float(G['mixdom1_ll']))
    for k in names:
        if k != 't':
            _close(v[k].grad, G[f'mixdom1_ct_{k}'], ('mixdom1', k))
    _close(v['t'].grad, G['mixdom1_g_t'], ('mixdom1', 't'))
    _close(v['Q'].grad, G['mixdom1_g_Q'], ('mixdom1', 'Q'))
    _close(v['pi'].grad, G['mixdom1_g_pi'], ('mixdom1', 'pi'))


@pytest.mark.parametrize('name', ['mixdom2_k3f1c1', 'mixdom2_k2f2c2'])
def test_mixdom2_log_prob_gradients(cuda_lib, name):
    from pairhmm import api
    keys = ['main_ins', 'main_del', 't', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates',
            'class_pis', 'class_S_exch', 'classdist']
    v = {k: _t(G[f'{name}_p_{k}']) for k in keys}
    x, y = G[f'{name}_x'].astype(np.int64), G[f'{name}_y'].astype(np.int64)
    ll = api.mixdom2_log_prob(*[v[k] for k in keys], x, y)
    ll.backward()
    want_ll = float(G[f'{name}_ll'])
    assert abs(float(ll.detach()) - want_ll) <= LL_RTOL * abs(want_ll)
    for k in keys[:8]:
        if k != 't':
            _close(v[k].grad, G[f'{name}_ct_{k}'], (name, k))
    _close(v['t'].grad, G[f'{name}_g_t'], (name, 't'))
    _close(v['class_S_exch'].grad, G[f'{name}_g_class_S_exch'], (name, 'class_S_exch'))
    _close(v['class_pis'].grad, G[f'{name}_g_class_pis'], (name, 'class_pis'))
    _close(v['classdist'].grad, G[f'{name}_g_classdist'], (name, 'classdist'))
