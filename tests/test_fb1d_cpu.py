"""1D alignment-conditioned forward-backward: the oracle restatement against
the reference's own outputs (tests/golden/fb1d.npz, make_golden_fb1d.py):
constrained per-class emissions, log P, posteriors and expected transitions
of forward_backward_1d_padded (sequential and associative scans agree)."""
import numpy as np
import pytest

from conftest import load_golden

CASES = ('k2f1c2', 'k3f1c1', 'k2f2c3', 'k1f1c1_short')


@pytest.mark.parametrize('name', CASES)
def test_oracle_matches_reference(name):
    from oracle import fb1d
    g = load_golden('fb1d')
    pre = name + '_'
    p = {k[len(pre) + 2:]: g[k] for k in g if k.startswith(pre + 'p_')}
    K, F = len(p['dom_ins']), p['frag_weights'].shape[1]
    le = fb1d.constrained_emissions_per_class(g[pre + 'state_types'], g[pre + 'cols'], g[pre + 'anc'],
                                              g[pre + 'desc'], g[pre + 'csubs'], p['class_pis'], p['classdist'],
                                              K, F)
    want = g[pre + 'log_emit']
    fin = want > -1e29
    assert (le[~fin] < -1e29).all()
    np.testing.assert_allclose(le[fin], want[fin], rtol=0, atol=1e-12)
    lp, post, n = fb1d.estep_1d(g[pre + 'chi'], g[pre + 'state_types'], g[pre + 'cols'], g[pre + 'anc'],
                                g[pre + 'desc'], g[pre + 'csubs'], p['class_pis'], p['classdist'], K, F,
                                int(g[pre + 'e_idx']))
    L = len(g[pre + 'cols'])
    assert abs(lp - g[pre + 'log_prob']) <= 1e-12 * abs(g[pre + 'log_prob'])
    np.testing.assert_allclose(post, g[pre + 'posteriors'][:L], atol=1e-12)
    np.testing.assert_allclose(n, g[pre + 'expected_trans'], atol=1e-11)
    assert abs(n.sum() - (L + 1)) < 1e-9   # initial + interior + terminal transitions
