"""The float64 oracle of the masked 2D forward-backward variants
(oracle/masked.py) against the reference's own outputs
(tests/golden/masked.npz): forward_backward_2d_banded around an MSA guide and
forward_backward_2d on a match-aligned emission table."""
import numpy as np
import pytest

from conftest import load_golden

BANDED = ('band_tkf91_a', 'band_tkf91_b', 'band_mixdom_a', 'band_tkf91_c')
MATCH = ('match_tkf91_a', 'match_mixdom_a', 'match_tkf91_b')


def _emit(g, pre):
    from oracle import dp
    st = g[pre + 'state_types']
    EM, EI, ED = dp.group_tables_tkf(g[pre + 'sub'], g[pre + 'pi'])
    return dp.log_emission_table(st, np.zeros(st.size, int), g[pre + 'x'], g[pre + 'y'], EM, EI, ED)


@pytest.mark.parametrize('name', BANDED)
def test_banded_oracle_matches_reference(name):
    from oracle import masked
    g = load_golden('masked')
    pre = name + '_'
    ll, post, n = masked.forward_backward_banded(g[pre + 'log_trans'], g[pre + 'state_types'], _emit(g, pre),
                                                 g[pre + 'band_center'], int(g[pre + 'band_width']))
    assert abs(ll - g[pre + 'log_prob']) <= 1e-12 * abs(g[pre + 'log_prob'])
    assert post.shape == g[pre + 'posteriors'].shape
    np.testing.assert_allclose(post, g[pre + 'posteriors'], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(n, g[pre + 'expected_trans'], rtol=1e-9, atol=1e-12)


def test_banded_reference_off_bin_rows():
    """Lx = 18 is not a padding bin (pad_to_bin(18) = 21): the reference's
    log-probability is the banded model's, its counts are not (their total is
    about 1 for a path of at least 22 steps); the oracle's counts add up to
    the expected path length."""
    from oracle import masked
    g = load_golden('masked')
    pre = 'band_tkf91_d_'
    ll, post, n = masked.forward_backward_banded(g[pre + 'log_trans'], g[pre + 'state_types'], _emit(g, pre),
                                                 g[pre + 'band_center'], int(g[pre + 'band_width']))
    assert abs(ll - g[pre + 'log_prob']) <= 1e-12 * abs(g[pre + 'log_prob'])
    assert g[pre + 'expected_trans'].sum() < 2.0
    assert n.sum() >= len(g[pre + 'y']) + 1 - 1e-9


@pytest.mark.parametrize('name', MATCH)
def test_match_aligned_oracle_matches_reference(name):
    from oracle import dp, masked
    g = load_golden('masked')
    pre = name + '_'
    st = g[pre + 'state_types']
    le = masked.mask_emissions_match_aligned(_emit(g, pre), st, g[pre + 'match_i'], g[pre + 'match_j'])
    ref = g[pre + 'log_emit']
    fin = ref > -1e29
    assert np.array_equal(fin, le > -1e29)
    np.testing.assert_allclose(le[fin], ref[fin], rtol=1e-13, atol=1e-13)
    ll, post, n, _, _ = dp.forward_backward(g[pre + 'log_trans'], st, le)
    assert abs(ll - g[pre + 'log_prob']) <= 1e-12 * abs(g[pre + 'log_prob'])
    gp = g[pre + 'posteriors']
    np.testing.assert_allclose(post, gp[:post.shape[0], :post.shape[1]], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(n, g[pre + 'expected_trans'], rtol=1e-9, atol=1e-12)
