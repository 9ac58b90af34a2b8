"""2D Viterbi oracle against the reference's own viterbi_2d outputs
(tests/golden/viterbi.npz, make_golden_viterbi.py)."""
import numpy as np
import pytest

from conftest import load_golden

CASES = ('tkf91_a', 'tkf91_b', 'tkf91_e', 'mixdom_a')


@pytest.mark.parametrize('name', CASES)
def test_oracle_matches_reference(name):
    from oracle import viterbi
    g = load_golden('viterbi')
    pre = name + '_'
    lp, path = viterbi.viterbi_2d(g[pre + 'log_trans'], g[pre + 'state_types'], g[pre + 'x'], g[pre + 'y'],
                                  g[pre + 'sub'], g[pre + 'pi'])
    assert abs(lp - g[pre + 'log_prob']) <= 1e-12 * abs(g[pre + 'log_prob'])
    assert np.array_equal(np.asarray(path), g[pre + 'path'])
