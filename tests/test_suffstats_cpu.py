"""Exact MixDom2 sufficient statistics (count restoration on the fully
exploded model) against the reference's own outputs (tests/golden,
make_golden_suffstats.py): the oracle restatement and the product's batched
torch implementation, both float64.  Bar: 1e-12 relative to each output's
largest entry."""
import numpy as np
import pytest
import torch

from conftest import load_golden

CASES = ('k2f1', 'k3f2', 'k2f2x', 'k2f1eq')
KEYS = ('top_5x5', 'dom_M_5x5', 'dom_kappa', 'dom_1mkappa', 'ext', 'term', 'dom_w', 'frag_w')


def case(name):
    g = load_golden('exact_suffstats')
    p = {k[len(name) + 3:]: g[k] for k in g if k.startswith(name + '_p_')}
    return g, p, g[name + '_t'], g[name + '_n_chi']


def close(got, want, tol=1e-12):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape
    assert np.abs(got - want).max() <= tol * max(np.abs(want).max(), 1e-300)


@pytest.mark.parametrize('name', CASES)
def test_oracle_matches_reference(name):
    from oracle import suffstats as osf
    g, p, ts, n = case(name)
    for b in range(len(ts)):
        ss = osf.exact_suffstats(n[b], p['main_ins'], p['main_del'], ts[b], p['dom_ins'], p['dom_del'],
                                 p['dom_weights'], p['frag_weights'], p['ext_rates'])
        for k in KEYS:
            close(ss[k], g[name + '_ss_' + k][b])


@pytest.mark.parametrize('name', CASES)
def test_batched_product_matches_reference(name):
    from pairhmm import suffstats
    g, p, ts, n = case(name)
    out = suffstats.exact_suffstats_batch(torch.as_tensor(n), p['main_ins'], p['main_del'], ts, p['dom_ins'],
                                          p['dom_del'], p['dom_weights'], p['frag_weights'], p['ext_rates'])
    for k in KEYS:
        v = out[k]
        got = torch.stack(v, dim=1).numpy() if isinstance(v, list) else v.numpy()
        close(got, g[name + '_bs_' + k])


def test_restored_chi_equals_collapsed_chi():
    """Eliminating the exploded model's null states gives the collapsed chi."""
    from oracle import suffstats as osf, models as om
    g, p, ts, n = case('k3f2')
    T, X = osf.build_exploded(p['main_ins'], p['main_del'], ts[0], p['dom_ins'], p['dom_del'],
                              p['dom_weights'], p['frag_weights'], p['ext_rates'])
    _, Tred = osf.restore(n[0], T, X)
    chi = om.build_nested_trans(p['main_ins'], p['main_del'], ts[0], p['dom_ins'], p['dom_del'],
                                p['dom_weights'], p['frag_weights'], p['ext_rates'])
    chi = chi[0] if isinstance(chi, tuple) else chi
    np.testing.assert_allclose(Tred, chi, atol=1e-15)
