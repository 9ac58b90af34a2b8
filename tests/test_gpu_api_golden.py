"""Public API (pairhmm.api) on the GPU against golden outputs of the
reference's own code (tests/golden, produced by make_golden.py).

Bars: log-likelihood 1e-6 relative, expected counts 1e-5 relative, as the
float32 DP is compared with the reference's float64 outputs.
"""
import numpy as np
import pytest
import torch

from conftest import load_golden, golden_params

pytestmark = pytest.mark.gpu
LL_RTOL = 1e-6
CNT_RTOL = 1e-5


def rel_close(got, want, rtol, floor=1e-6):
    got = np.asarray(got, float)
    want = np.asarray(want, float)
    scale = max(np.abs(want).max(), 1e-300)
    sig = np.abs(want) > floor * scale
    if sig.any():
        rel = np.abs(got[sig] - want[sig]) / np.abs(want[sig])
        assert rel.max() < rtol, f'max rel err {rel.max():.3e}'
    assert np.abs(got - want).max() <= rtol * scale + 1e-12


def log_close(got, want, rtol=LL_RTOL):
    """log tables: finite entries relative; NEG_INF-like entries both tiny."""
    got = np.asarray(got)
    want = np.asarray(want)
    fin = want > -1e29
    assert (got[~fin] < -1e29).all()
    np.testing.assert_allclose(got[fin], want[fin], rtol=rtol, atol=1e-5)


@pytest.mark.parametrize('name', ['tkf91', 'tkf92', 'tkf91_wild'])
def test_tkf_api_matches_reference(cuda_lib, name):
    from pairhmm import api
    from pairhmm import models as pm
    g = load_golden(name)
    p = golden_params(g)
    model = str(g['model'])
    x, y = g['x'], g['y']
    lt = np.log(np.where(g['chi'] > 0, g['chi'], 1.0))
    lt[g['chi'] <= 0] = -1e30
    st = np.array([0, 1, 2, 3, 4])
    ll, F = api.forward_2d(lt, st, x, y, g['sub'], p['pi'])
    assert abs(ll - g['ll_forward']) <= LL_RTOL * abs(g['ll_forward'])
    log_close(F, g['F'])
    B = api.backward_2d(lt, st, x, y, g['sub'], p['pi'])
    log_close(B[:, :, :4], g['B'][:, :, :4])      # E-row of B is NEG_INF in both
    ll2, post, n = api.forward_backward_2d(lt, st, x, y, g['sub'], p['pi'])
    assert post.shape == (api.pad_to_bin(len(x)) + 1, api.pad_to_bin(len(y)) + 1, 5)
    rel_close(post[:len(x) + 1, :len(y) + 1], g['post'], CNT_RTOL)
    rel_close(n, g['n_trans'], CNT_RTOL)
    ll3, n3, ss = api.e_step(model, p, x, y)
    assert abs(ll3 - g['ll_estep']) <= LL_RTOL * abs(g['ll_estep'])
    rel_close(n3, g['n_estep'], CNT_RTOL)
    for k, v in ss['pi_obs_counts'].items():
        rel_close(v, g['obs_' + k], CNT_RTOL)
    mp = np.array(ss['match_pairs'], float).reshape(-1, 3)
    ref = g['match_pairs']
    # same (a, b) cells above the 1e-8 threshold, weights within tolerance
    key = lambda a: {(int(r[0]), int(r[1]), round(r[2], 4)) for r in a}
    assert abs(len(mp) - len(ref)) <= 2
    rel_close(np.sort(mp[:, 2]), np.sort(ref[:, 2]), 1e-4) if len(mp) == len(ref) else None


@pytest.mark.parametrize('name', ['mixdom2_k3f1c1', 'mixdom2_k2f2c2', 'mixdom2_k1f2c3_wild'])
def test_e_step_mixdom2_matches_reference(cuda_lib, name):
    from pairhmm import api
    g = load_golden(name)
    p = golden_params(g)
    ll, n, ss = api.e_step_mixdom2(p, g['x'], g['y'])
    assert abs(ll - g['ll']) <= LL_RTOL * abs(g['ll'])
    rel_close(n, g['n_trans'], CNT_RTOL)
    for k, v in ss.items():
        rel_close(v, g['ss_' + k], CNT_RTOL)


def test_forward_backward_with_log_emit_table_mixdom1(cuda_lib):
    """MixDom1 per-domain emission table passed as log_emit_table (train_pfam.py:1705-1710)."""
    from pairhmm import api
    g = load_golden('mixdom1_d3f2')
    K, F = int(g['K']), int(g['F'])
    from pairhmm import models as pm
    st = pm.mixdom_state_types(K, F)
    lt = np.where(g['chi'] > 0, np.log(np.where(g['chi'] > 0, g['chi'], 1.0)), -1e30)
    ll, post, n = api.forward_backward_2d(lt, st, g['x'], g['y'], None, None,
                                          log_emit_table=g['log_emit'])
    assert abs(ll - g['ll']) <= LL_RTOL * abs(g['ll'])
    rel_close(post[:len(g['x']) + 1, :len(g['y']) + 1], g['post'], CNT_RTOL)
    rel_close(n, g['n_trans'], CNT_RTOL)


def test_batched_tkf92_forward_only(cuda_lib):
    from pairhmm import api
    g = load_golden('batch_tkf92_fwd')
    lp = api.estep_batch_tkf92_forward_only(g['xs'], g['ys'], g['ts'], g['Lx'], g['Ly'],
                                            float(g['lam']), float(g['mu']), float(g['ext']),
                                            g['Q'], g['pi']).cpu().numpy()
    np.testing.assert_allclose(lp, g['log_p'], rtol=LL_RTOL)


def test_batched_tkf92_estep_bdi_statistics(cuda_lib):
    """estep_batch_tkf92's full dict (log_p, BDI B/D/S, L, M, T, extension
    counts) against the oracle E-step and its float64 epilogue."""
    from pairhmm import api
    from oracle import estep as oe, bdi as ob
    g = load_golden('batch_tkf92_fwd')
    lam, mu, ext = float(g['lam']), float(g['mu']), float(g['ext'])
    r = api.estep_batch_tkf92(g['xs'], g['ys'], g['ts'], g['Lx'], g['Ly'], lam, mu, ext, g['Q'], g['pi'])
    r = {k: v.cpu().numpy() for k, v in r.items()}
    for b in range(len(g['ts'])):
        x = np.asarray(g['xs'][b])[:int(g['Lx'][b])]
        y = np.asarray(g['ys'][b])[:int(g['Ly'][b])]
        p = {'ins_rate': lam, 'del_rate': mu, 't': float(g['ts'][b]), 'ext': ext, 'Q': g['Q'], 'pi': g['pi']}
        ll, n, _ = oe.e_step('tkf92', p, x, y)
        assert abs(r['log_p'][b] - ll) <= LL_RTOL * abs(ll)
        want = ob.tkf92_epilogue(n, lam, mu, float(g['ts'][b]), ext)
        for k, w in want.items():
            assert abs(r[k][b] - w) <= CNT_RTOL * max(abs(w), 1.0), (k, b, r[k][b], w)
        assert r['T'][b] == g['ts'][b]


def test_empty_sequences(cuda_lib):
    from pairhmm import api
    g = load_golden('edges_tkf91')
    lt = np.where(g['chi'] > 0, np.log(np.where(g['chi'] > 0, g['chi'], 1.0)), -1e30)
    st = np.array([0, 1, 2, 3, 4])
    for tag in ('x0', 'y0', 'xy0', 'x1y1'):
        x, y = g[f'{tag}_x'], g[f'{tag}_y']
        ll, post, n = api.forward_backward_2d(lt, st, x, y, g['sub'], g['pi'])
        assert abs(ll - g[f'{tag}_ll']) <= LL_RTOL * abs(g[f'{tag}_ll']), tag
        rel_close(n, g[f'{tag}_n'], CNT_RTOL)


def test_mixdom2_gradient_vs_oracle_finite_differences(cuda_lib):
    """d(sum LL)/d(theta) through the autograd adjoint vs central FD of the
    FP64 oracle (h = 1e-6 relative)."""
    from pairhmm import api
    from oracle import models as om, dp as odp, estep as oe
    g = load_golden('mixdom2_k2f2c2')
    p = golden_params(g)
    x, y = g['x'], g['y']
    names = ['main_ins', 'main_del', 't', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights',
             'ext_rates', 'class_pis', 'class_S_exch', 'classdist']
    tens = {k: torch.tensor(np.asarray(p[k], float), dtype=torch.float64, requires_grad=True)
            for k in names}
    ll = api.mixdom2_log_prob(tens['main_ins'], tens['main_del'], tens['t'], tens['dom_ins'],
                              tens['dom_del'], tens['dom_weights'], tens['frag_weights'],
                              tens['ext_rates'], tens['class_pis'], tens['class_S_exch'],
                              tens['classdist'], x, y)
    ll.backward()

    def oracle_ll(pp):
        chi, st, groups, EM, EI, ED, _ = oe.mixdom2_model(pp)
        emit = odp.log_emission_table(st, groups, x, y, EM, EI, ED)
        return odp.forward_table(om.safe_log(chi), st, emit)[0]
    rng = np.random.default_rng(0)
    for k in names:
        v = np.asarray(p[k], float)
        flat = v.reshape(-1)
        for idx in rng.choice(flat.size, size=min(3, flat.size), replace=False):
            h = 1e-6 * max(abs(flat[idx]), 1e-3)
            pp, pm_ = dict(p), dict(p)
            a = flat.copy(); a[idx] += h
            b = flat.copy(); b[idx] -= h
            pp[k] = a.reshape(v.shape) if v.ndim else float(a[0])
            pm_[k] = b.reshape(v.shape) if v.ndim else float(b[0])
            fd = (oracle_ll(pp) - oracle_ll(pm_)) / (2 * h)
            got = tens[k].grad.numpy().reshape(-1)[idx]
            assert abs(got - fd) <= 2e-4 * max(abs(fd), 1.0), (k, idx, got, fd)
