"""The float64 oracle of the beam-pruned forward-backward (oracle/beam.py)
against the reference's own dp/hmm_beam.py outputs (tests/golden/beam.npz)."""
import numpy as np
import pytest

from conftest import load_golden

CASES = ('tkf91_env', 'tkf91_beam', 'tkf91_both', 'mixdom_both', 'mixdom_beam')


@pytest.mark.parametrize('name', CASES)
def test_beam_oracle_matches_reference(name):
    from oracle import beam
    g = load_golden('beam')
    pre = name + '_'
    env = None
    if pre + 'envelope' in g:
        env = beam.msa_to_envelope(len(g[pre + 'x']), len(g[pre + 'y']), g[pre + 'msa_x'], g[pre + 'msa_y'],
                                   int(g[pre + 'band_width']))
        assert np.array_equal(env, g[pre + 'envelope'])
    args = (g[pre + 'log_trans'], g[pre + 'state_types'], g[pre + 'x'], g[pre + 'y'], g[pre + 'sub'], g[pre + 'pi'],
            float(g[pre + 'beam']), env)
    lp, F, n_cells = beam.beam_forward(*args)
    assert n_cells == int(g[pre + 'n_cells'])
    lp2, post, F2 = beam.beam_forward_backward(*args)
    assert lp == lp2
    assert abs(lp - g[pre + 'log_prob']) <= 1e-12 * abs(g[pre + 'log_prob'])
    live = g[pre + 'F'] > -1e29
    assert np.array_equal(live, F > -1e29)
    np.testing.assert_allclose(F[live], g[pre + 'F'][live], rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(post, g[pre + 'posteriors'], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize('name', CASES)
def test_beam_viterbi_oracle_matches_reference(name):
    from oracle import beam
    g = load_golden('beam')
    pre = name + '_'
    env = g[pre + 'envelope'] if pre + 'envelope' in g else None
    lp, path = beam.beam_viterbi(g[pre + 'log_trans'], g[pre + 'state_types'], g[pre + 'x'], g[pre + 'y'],
                                 g[pre + 'sub'], g[pre + 'pi'], env)
    assert lp == float(g[pre + 'viterbi_log_prob'])
    assert np.array_equal(np.asarray(path), g[pre + 'viterbi_path'])
