"""1D alignment-conditioned forward-backward on the GPU (phmm_fb1d,
phmm_fb1d_emissions) against the reference's outputs (tests/golden/fb1d.npz)
and the float64 oracle.  Bars: log P 1e-6 relative; posteriors 1e-5
absolute; expected transitions 1e-5 relative to the largest entry (the
float32 DP's bars)."""
import numpy as np
import pytest
import torch

from conftest import load_golden

pytestmark = pytest.mark.gpu
CASES = ('k2f1c2', 'k3f1c1', 'k2f2c3', 'k1f1c1_short')


def params_of(g, pre):
    p = {k[len(pre) + 2:]: g[k] for k in g if k.startswith(pre + 'p_')}
    return p


def test_generic_batch_matches_reference(cuda_lib):
    """forward_backward_1d_batch on the reference's own log emissions, all cases padded into one batch."""
    from pairhmm import api
    g = load_golden('fb1d')
    for name in CASES:
        pre = name + '_'
        Lp = int(g[pre + 'Lpad'])
        L = len(g[pre + 'cols'])
        le = np.full((2, Lp, g[pre + 'log_emit'].shape[1]), -1e30)
        le[0, :L] = g[pre + 'log_emit']
        le[1, :L] = g[pre + 'log_emit']
        lt = np.log(np.where(g[pre + 'chi'] > 0, g[pre + 'chi'], 1e-300))
        lt[g[pre + 'chi'] <= 0] = -1e30
        lp, post, nt = api.forward_backward_1d_batch(lt, le, [L, L], 0, int(g[pre + 'e_idx']))
        want = g[pre + 'log_prob']
        for b in range(2):
            assert abs(lp[b].item() - want) <= 1e-6 * abs(want)
            np.testing.assert_allclose(post[b].cpu().numpy(), g[pre + 'posteriors'], atol=1e-5)
            n = nt[b].cpu().numpy()
            scale = np.abs(g[pre + 'expected_trans']).max()
            assert np.abs(n - g[pre + 'expected_trans']).max() <= 1e-5 * scale


def test_mixdom2_alignment_estep_matches_reference(cuda_lib):
    """estep_1d_mixdom2: device prologue + constrained emissions + 1D FB."""
    from pairhmm import api
    g = load_golden('fb1d')
    for name in CASES:
        pre = name + '_'
        p = params_of(g, pre)
        res = api.estep_1d_mixdom2(p, [g[pre + 'cols']], [g[pre + 'anc']], [g[pre + 'desc']],
                                   np.array([float(g[pre + 't'])]), with_posteriors=True)
        want = g[pre + 'log_prob']
        assert abs(res['log_p'][0].item() - want) <= 1e-6 * abs(want), name
        assert int(res['status'][0]) == 0
        n = res['n_trans'][0].cpu().numpy()
        assert np.abs(n - g[pre + 'expected_trans']).max() <= 1e-5 * np.abs(g[pre + 'expected_trans']).max()
        L = len(g[pre + 'cols'])
        np.testing.assert_allclose(res['posteriors'][0].cpu().numpy(), g[pre + 'posteriors'][:L], atol=1e-5)


def test_random_alignments_against_oracle(cuda_lib):
    """Ragged batch (lengths 0, 1, ... 700) against the float64 oracle."""
    from pairhmm import api, synth
    from pairhmm import models as pm
    from oracle import fb1d, models as om
    rng = np.random.default_rng(91)
    K, F, C = 3, 2, 2
    p = synth.mixdom2_params(rng, K, F, C)
    lens = [0, 1, 2, 37, 150, 700]
    cols = [rng.choice(np.array([1, 2, 3]), size=n, p=[0.6, 0.2, 0.2]).astype(np.uint8) for n in lens]
    ancs = [rng.integers(0, 21, n).astype(np.uint8) for n in lens]
    descs = [rng.integers(0, 21, n).astype(np.uint8) for n in lens]
    ts = np.exp(rng.uniform(-2, 0.5, len(lens)))
    res = api.estep_1d_mixdom2(p, cols, ancs, descs, ts)
    st = pm.mixdom_state_types(K, F)
    for b in range(len(lens)):
        chi = om.build_nested_trans(p['main_ins'], p['main_del'], ts[b], p['dom_ins'], p['dom_del'],
                                    p['dom_weights'], p['frag_weights'], p['ext_rates'])
        csubs = om.build_class_subs(p['class_S_exch'], p['class_pis'], ts[b])
        lp, _, n = fb1d.estep_1d(chi, st, cols[b], ancs[b], descs[b], csubs, p['class_pis'], p['classdist'], K, F)
        assert abs(res['log_p'][b].item() - lp) <= 1e-6 * abs(lp), (b, res['log_p'][b].item(), lp)
        got = res['n_trans'][b].cpu().numpy()
        assert np.abs(got - n).max() <= 1e-5 * np.abs(n).max(), b


def test_constrained_log_prob_gradient_against_fd(cuda_lib):
    """mixdom2_constrained_log_prob: log P and every parameter's gradient
    against the float64 oracle (central differences, h = 1e-6 relative)."""
    from pairhmm import api, synth
    from pairhmm import models as pm
    from oracle import fb1d, models as om
    rng = np.random.default_rng(93)
    K, F, C = 2, 2, 2
    p = synth.mixdom2_params(rng, K, F, C)
    L = 60
    cols = rng.choice(np.array([1, 2, 3]), size=L, p=[0.6, 0.2, 0.2])
    anc = rng.integers(0, 20, L)
    desc = rng.integers(0, 20, L)
    names = ['main_ins', 'main_del', 't', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates',
             'class_S_exch', 'class_pis', 'classdist']
    tens = {k: torch.tensor(np.asarray(p[k], float), dtype=torch.float64, requires_grad=True) for k in names}
    ll = api.mixdom2_constrained_log_prob(*[tens[k] for k in names], cols, anc, desc, L)
    ll.backward()
    st = pm.mixdom_state_types(K, F)

    def oracle_ll(q):
        chi = om.build_nested_trans(q['main_ins'], q['main_del'], q['t'], q['dom_ins'], q['dom_del'],
                                    q['dom_weights'], q['frag_weights'], q['ext_rates'])
        cs = om.build_class_subs(q['class_S_exch'], q['class_pis'], q['t'])
        return fb1d.estep_1d(chi, st, cols, anc, desc, cs, q['class_pis'], q['classdist'], K, F)[0]
    want = oracle_ll(p)
    assert abs(ll.item() - want) <= 1e-6 * abs(want)
    for k in names:
        v = np.asarray(p[k], float)
        flat = v.reshape(-1)
        for idx in rng.choice(flat.size, size=min(2, flat.size), replace=False):
            if k == 'class_S_exch':   # only off-diagonal exchangeabilities enter Q
                a_, b_ = divmod(int(idx) % 400, 20)
                if a_ == b_:
                    continue
            h = 1e-6 * max(abs(flat[idx]), 1e-3)
            pp, pm_ = dict(p), dict(p)
            a = flat.copy(); a[idx] += h
            b = flat.copy(); b[idx] -= h
            pp[k] = a.reshape(v.shape) if v.ndim else float(a[0])
            pm_[k] = b.reshape(v.shape) if v.ndim else float(b[0])
            fd = (oracle_ll(pp) - oracle_ll(pm_)) / (2 * h)
            got = tens[k].grad.numpy().reshape(-1)[idx]
            assert abs(got - fd) <= 2e-4 * max(abs(fd), 1.0), (k, idx, got, fd)
