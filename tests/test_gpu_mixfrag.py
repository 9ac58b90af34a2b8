"""MixFrag batched E-step and the TKF92 Adam log-likelihood on the GPU against
the reference's own outputs (tests/golden/mixfrag.npz from
train/mixfrag_svi_bw.py:194-250 and train/tkf92_adam_fb.py:77-104).

The MixFrag state spaces with F = 2 and F = 3 fragment types (8 and 11
states) run on the two-warp stripe kernels (the automatic choice for their
shapes).  Bars: log-likelihood 1e-6 relative; the count-derived statistics
(F_f, E_f, L, M, and B, D, S after the float64 BDI epilogue) 1e-5 relative
to max(|v|, 1e-3)."""
import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
G = np.load(GOLDEN + '/mixfrag.npz')
LL_RTOL = 1e-6
CNT_RTOL = 1e-5


def _args(name):
    return (G[f'{name}_xs'], G[f'{name}_ys'], G[f'{name}_ts'], G[f'{name}_Lx'], G[f'{name}_Ly'],
            float(G[f'{name}_lam']), float(G[f'{name}_mu']), G[f'{name}_exts'], G[f'{name}_weights'],
            G[f'{name}_Q'], G[f'{name}_pi'])


@pytest.mark.parametrize('name', ['f2', 'f3'])
def test_estep_batch_mixfrag_matches_reference(cuda_lib, name):
    from pairhmm import api
    from pairhmm import models as pm
    res = api.estep_batch_mixfrag(*_args(name))
    torch.cuda.synchronize()
    F = G[f'{name}_exts'].size
    plan = api.get_plan(pm.mixfrag_state_types(F), np.zeros(3 * F + 2, np.int32), 1)
    assert plan.last_variant == 7   # two-warp stripes
    assert (res['status'].cpu().numpy() == 0).all()
    want = G[f'{name}_out_log_p']
    got = res['log_p'].cpu().numpy()
    assert np.all(np.abs(got - want) <= LL_RTOL * np.abs(want)), (got, want)
    for k in ('B', 'D', 'S', 'L', 'M', 'T', 'F_f', 'E_f'):
        g = res[k].cpu().numpy()
        w = G[f'{name}_out_{k}']
        err = np.abs(g - w) / np.maximum(np.abs(w), 1e-3)
        assert err.max() <= CNT_RTOL, (k, g, w)
    fwd = api.estep_batch_mixfrag_forward_only(*_args(name)).cpu().numpy()
    assert np.all(np.abs(fwd - G[f'{name}_fwd_log_p']) <= LL_RTOL * np.abs(G[f'{name}_fwd_log_p']))


def test_tkf92_log_prob_fb_value_and_gradient(cuda_lib):
    """Value against the reference (padded and not); gradient in lam, mu, ext,
    t against central differences of the FP64 oracle."""
    from pairhmm import api
    from oracle import models as om, dp as odp
    v = {k: torch.tensor(float(G[f'fb_{k}']), dtype=torch.float64, requires_grad=True)
         for k in ('lam', 'mu', 'ext', 't')}
    Q, pi = G['fb_Q'], G['fb_pi']
    ll = api.tkf92_log_prob_fb(v['lam'], v['mu'], v['ext'], v['t'], Q, pi, G['fb_x'], G['fb_y'])
    ll.backward()
    want = float(G['fb_log_p'])
    assert abs(float(ll.detach()) - want) <= LL_RTOL * abs(want)
    llp = api.tkf92_log_prob_fb(float(G['fb_lam']), float(G['fb_mu']), float(G['fb_ext']), float(G['fb_t']), Q, pi,
                                G['fb_xp'], G['fb_yp'], real_Lx=G['fb_x'].size, real_Ly=G['fb_y'].size)
    assert abs(float(llp) - float(G['fb_log_p_padded'])) <= LL_RTOL * abs(want)
    x, y = G['fb_x'].astype(int), G['fb_y'].astype(int)

    def oracle_ll(q):
        chi = np.maximum(om.tkf92_trans(q['lam'], q['mu'], q['t'], q['ext']), 1e-30)
        EM, EI, ED = odp.group_tables_tkf(om.transition_matrix(Q, q['t']), pi)
        st = om.tkf_state_types()
        return odp.forward_table(om.safe_log(chi), st, odp.log_emission_table(st, np.zeros(5, int), x, y, EM, EI,
                                                                             ED))[0]
    q0 = {k: float(G[f'fb_{k}']) for k in ('lam', 'mu', 'ext', 't')}
    for k in q0:
        h = 1e-6 * abs(q0[k])
        fd = (oracle_ll(dict(q0, **{k: q0[k] + h})) - oracle_ll(dict(q0, **{k: q0[k] - h}))) / (2 * h)
        assert abs(float(v[k].grad) - fd) <= 2e-5 * max(abs(fd), 1.0), (k, float(v[k].grad), fd)
