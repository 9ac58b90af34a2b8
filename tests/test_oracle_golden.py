"""The FP64 oracle against golden outputs of the reference's own code.

The fixtures in tests/golden were produced by running the unmodified
reference modules (dp/hmm.py, models/mixdom.py, train/likelihood.py,
train/vjp.py, train/tkf92_svi_bw.py) under a NumPy stand-in for JAX
(tests/golden/make_golden.py).  Bar: 1e-11 relative (float64 restatement).
"""
import numpy as np
import pytest

from conftest import load_golden, golden_params
from oracle import models as om, dp as odp, estep as oe

RTOL = 1e-11


def close(a, b, rtol=RTOL, atol=1e-13):
    np.testing.assert_allclose(np.asarray(a, float), np.asarray(b, float), rtol=rtol, atol=atol)


@pytest.mark.parametrize('name', ['tkf91', 'tkf92', 'tkf91_wild'])
def test_tkf_tables_and_estep(name):
    g = load_golden(name)
    p = golden_params(g)
    model = str(g['model'])
    x, y = g['x'], g['y']
    chi, st, groups, EM, EI, ED, sub = oe.tkf_model(model, p)
    close(chi, g['chi'])
    close(sub, g['sub'])
    emit = odp.log_emission_table(st, groups, x, y, EM, EI, ED)
    ll, post, n, F, B = odp.forward_backward(om.safe_log(chi), st, emit)
    close(ll, g['ll_forward'])
    close(ll, g['ll_fb'])
    close(F, g['F'], atol=1e-9)
    close(B, g['B'], atol=1e-9)
    close(post, g['post'])
    close(n, g['n_trans'])
    ll_e, n_e, ss = oe.e_step(model, p, x, y)
    close(ll_e, g['ll_estep'])
    close(n_e, g['n_estep'])
    mp = np.array(ss['match_pairs'], float).reshape(-1, 3)
    close(mp, g['match_pairs'])
    for k, v in ss['pi_obs_counts'].items():
        close(v, g['obs_' + k])


@pytest.mark.parametrize('name', ['mixdom2_k3f1c1', 'mixdom2_k2f2c2', 'mixdom2_k1f2c3_wild'])
def test_mixdom2_estep_and_vjp_counts(name):
    g = load_golden(name)
    p = golden_params(g)
    x, y = g['x'], g['y']
    chi, st, groups, EM, EI, ED, cs = oe.mixdom2_model(p)
    close(chi, g['chi'])
    close(cs, g['class_subs'])
    emit = odp.log_emission_table(st, groups, x, y, EM, EI, ED)
    close(emit, g['log_emit'][:len(x) + 1, :len(y) + 1], atol=1e-12)
    ll, n, ss = oe.e_step_mixdom2(p, x, y)
    close(ll, g['ll'])
    close(ll, g['ll_dp'])
    close(ll, g['ll_fwd_only'])
    close(n, g['n_trans'])
    close(n, g['n_chi'])
    for k, v in ss.items():
        close(v, g['ss_' + k])
    _, post, _, _, _ = odp.forward_backward(om.safe_log(chi), st, emit)
    close(post, g['post'])
    cM, cI, cD = oe.char_count_tables(post, st, groups, x, y, EM.shape[0])
    mc, V, cdc = oe.mixdom2_emission_counts(p, cM, cI, cD)
    close(mc, g['mc_c'])
    close(V, g['V_c_linear'])
    close(cdc, g['cd_count'])


def test_mixdom1_trained_params_per_domain():
    g = load_golden('mixdom1_d3f2')
    K, F = int(g['K']), int(g['F'])
    chi = om.build_nested_trans(g['main_ins'], g['main_del'], float(g['t']), g['dom_ins'],
                                g['dom_del'], g['dom_weights'], g['frag_weights'],
                                g['ext_rates'])
    close(chi, g['chi'])
    subs = np.stack([om.transition_matrix(q, float(g['t'])) for q in g['dom_Qs']])
    close(subs, g['subs'])
    EM, EI, ED = odp.group_tables_per_domain(subs, g['dom_pis'], K)
    st = om.mixdom_state_types(K, F)
    dom_groups = np.concatenate([[0, 0], np.arange(5 * K * F) // (5 * F)])
    emit = odp.log_emission_table(st, dom_groups, g['x'], g['y'], EM, EI, ED)
    close(emit, g['log_emit'][:len(g['x']) + 1, :len(g['y']) + 1], atol=1e-12)
    ll, post, n, _, _ = odp.forward_backward(om.safe_log(chi), st, emit)
    close(ll, g['ll'])
    close(post, g['post'])
    close(n, g['n_trans'])


def test_builders():
    g = load_golden('builders')
    close(om.mixfrag_trans(0.02, 0.026, 0.8, [0.3, 0.7], [0.6, 0.4]), g['mixfrag'])
    close(om.tkf92_trans(0.02, 0.026, 0.8, 0.35), g['tkf92'])
    close(om.tkf91_trans(0.03, 0.03 * (1 + 3e-5), 0.9), g['tkf91_limit'])


@pytest.mark.parametrize('tag', ['x0', 'y0', 'xy0', 'x1y1'])
def test_empty_and_tiny_sequences(tag):
    g = load_golden('edges_tkf91')
    x, y = g[f'{tag}_x'], g[f'{tag}_y']
    EM, EI, ED = odp.group_tables_tkf(g['sub'], g['pi'])
    st = om.tkf_state_types()
    emit = odp.log_emission_table(st, np.zeros(5, int), x, y, EM, EI, ED)
    ll, post, n, _, _ = odp.forward_backward(om.safe_log(g['chi']), st, emit)
    close(ll, g[f'{tag}_ll'])
    close(n, g[f'{tag}_n'])
    close(post, g[f'{tag}_post'])


def test_batched_forward_with_padding():
    g = load_golden('batch_tkf92_fwd')
    chi = om.tkf92_trans(float(g['lam']), float(g['mu']), 0.0 + 1.0, float(g['ext']))
    for b in range(g['xs'].shape[0]):
        t = float(g['ts'][b])
        chi = om.tkf92_trans(float(g['lam']), float(g['mu']), t, float(g['ext']))
        # the batched reference path uses log(max(tau, 1e-30)) (tkf92_svi_bw.py:164)
        lt = np.log(np.maximum(chi, 1e-30))
        sub = om.transition_matrix(g['Q'], t)
        EM, EI, ED = odp.group_tables_tkf(sub, g['pi'])
        x = g['xs'][b, :g['Lx'][b]]
        y = g['ys'][b, :g['Ly'][b]]
        st = om.tkf_state_types()
        emit = odp.log_emission_table(st, np.zeros(5, int), x, y, EM, EI, ED)
        ll, _ = odp.forward_table(lt, st, emit)
        close(ll, g['log_p'][b])


def test_invariants_tkf92_ext0_is_tkf91_and_mixfrag_f1():
    close(om.tkf92_trans(0.02, 0.03, 0.7, 0.0), om.tkf91_trans(0.02, 0.03, 0.7))
    close(om.mixfrag_trans(0.02, 0.03, 0.7, [0.4], [1.0]), om.tkf92_trans(0.02, 0.03, 0.7, 0.4))


def test_count_conservation():
    """sum over M+D destinations = Lx, over M+I = Ly, n[:,E] sums to 1."""
    g = load_golden('mixdom2_k2f2c2')
    p = golden_params(g)
    x, y = g['x'], g['y']
    chi, st, groups, EM, EI, ED, _ = oe.mixdom2_model(p)
    emit = odp.log_emission_table(st, groups, x, y, EM, EI, ED)
    ll, post, n, F, B = odp.forward_backward(om.safe_log(chi), st, emit)
    colsum = n.sum(axis=0)
    close(colsum[(st == om.M) | (st == om.D)].sum(), len(x), rtol=1e-12)
    close(colsum[(st == om.M) | (st == om.I)].sum(), len(y), rtol=1e-12)
    close(n[:, 1].sum(), 1.0, rtol=1e-12)
    # forward and backward agree on the likelihood: B at the origin
    close(B[0, 0, 0], ll)
