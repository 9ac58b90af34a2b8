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


def _sample_paths(g, pre):
    lens = g[pre + 'sample_lens']
    rows = g[pre + 'sample_paths']
    return [rows[a:b] for a, b in zip(np.r_[0, np.cumsum(lens)[:-1]], np.cumsum(lens))]


@pytest.mark.parametrize('name', CASES)
def test_beam_sample_traceback_matches_reference_draws(name):
    """pairhmm.api.beam_sample_traceback on the reference's forward table with
    the reference's RandomState seed: the same four paths, draw for draw
    (host code of the drop-in; no GPU)."""
    from pairhmm import api
    g = load_golden('beam')
    pre = name + '_'
    env = g[pre + 'envelope'] if pre + 'envelope' in g else None
    rng = np.random.RandomState(int(g[pre + 'sample_seed']))
    for want in _sample_paths(g, pre):
        got = api.beam_sample_traceback(g[pre + 'log_trans'], g[pre + 'state_types'], g[pre + 'F'],
                                        float(g[pre + 'log_prob']), g[pre + 'x'], g[pre + 'y'], g[pre + 'sub'],
                                        g[pre + 'pi'], rng, env)
        assert np.array_equal(np.asarray(got, np.int64).reshape(-1, 3), want)
        assert got[0] == (0, 0, 0)


def test_beam_sample_traceback_unreachable_end_is_empty():
    from pairhmm import api
    st = np.array([0, 1, 2, 3, 4])
    F = np.full((3, 2, 5), -1e30)
    lt = np.zeros((5, 5))
    assert api.beam_sample_traceback(lt, st, F, -1e30, [1, 2], [3], None, None, np.random.RandomState(0)) == []
