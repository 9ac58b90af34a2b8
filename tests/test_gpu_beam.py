"""Beam-pruned forward-backward on the GPU (phmm_batch.beam_log_width and an
envelope cell mask, generic kernels) against the reference's own
dp/hmm_beam.py outputs (tests/golden/beam.npz): log-likelihood 1e-6
relative, the pruned forward table 1e-5 where it lives (float32 DP against
float64; the same cells live), posteriors 1e-5.  Iterative refinement
reproduces the reference's final envelope and likelihood."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu
CASES = ('tkf91_env', 'tkf91_beam', 'tkf91_both', 'mixdom_both', 'mixdom_beam')


def _args(g, pre):
    env = g[pre + 'envelope'] if pre + 'envelope' in g else None
    return (g[pre + 'log_trans'], g[pre + 'state_types'], g[pre + 'x'], g[pre + 'y'], g[pre + 'sub'],
            g[pre + 'pi'], float(g[pre + 'beam']), env)


@pytest.mark.parametrize('name', CASES)
def test_beam_forward_backward_matches_reference(cuda_lib, name):
    from pairhmm import api
    g = load_golden('beam')
    pre = name + '_'
    lp, post, F = api.beam_forward_backward_2d(*_args(g, pre))
    ref = float(g[pre + 'log_prob'])
    assert abs(lp - ref) <= 1e-6 * abs(ref)
    live = g[pre + 'F'] > -1e29
    assert np.array_equal(F > -1e29, live)
    np.testing.assert_allclose(F[live], g[pre + 'F'][live], rtol=1e-5, atol=1e-4)
    np.testing.assert_allclose(post, g[pre + 'posteriors'], rtol=1e-5, atol=1e-6)
    lp2, F2, n_cells = api.beam_forward_2d(*_args(g, pre))
    assert lp2 == lp and n_cells == int(g[pre + 'n_cells'])


def test_iterative_refinement_matches_reference(cuda_lib):
    from pairhmm import api
    g = load_golden('beam')
    lp, F, env = api.iterative_beam_refinement(g['refine_log_trans'], g['refine_state_types'], g['refine_x'],
                                               g['refine_y'], g['refine_sub'], g['refine_pi'], beam_log_width=8.0,
                                               initial_band=3, n_iterations=3, band_shrink=0.7)
    assert np.array_equal(env, g['refine_envelope'])
    assert abs(lp - float(g['refine_log_prob'])) <= 1e-6 * abs(float(g['refine_log_prob']))


def test_beam_refused_by_other_families(cuda_lib):
    from pairhmm import api, synth, _lib
    from oracle import dp, models as om
    rng = np.random.default_rng(4)
    Q, pi, _ = synth.rand_Q_pi(rng)
    chi = om.tkf91_trans(0.03, 0.035, 0.4)
    st = np.array([0, 1, 2, 3, 4], np.int8)
    EM, EI, ED = dp.group_tables_tkf(om.transition_matrix(Q, 0.4), pi)
    x, y = rng.integers(0, 20, 20), rng.integers(0, 20, 30)
    plan = api.get_plan(st, np.zeros(5, np.int32), 1)
    plan.set_variant(7)
    try:
        with pytest.raises(_lib.PairHMMError):
            _lib.estep(plan, _lib.make_batch([x], [y], chi[None], EM, EI, ED, beam_log_width=5.0))
    finally:
        plan.set_variant(0)
    out = _lib.estep(plan, _lib.make_batch([x], [y], chi[None], EM, EI, ED, beam_log_width=5.0))
    assert plan.last_variant == 1 and int(out['status'][0]) == 0


@pytest.mark.parametrize('name', CASES)
def test_beam_viterbi_matches_reference(cuda_lib, name):
    """Envelope-constrained Viterbi (float64 on the device): the reference's
    best path and its log-probability to 1e-12."""
    from pairhmm import api
    g = load_golden('beam')
    pre = name + '_'
    env = g[pre + 'envelope'] if pre + 'envelope' in g else None
    lp, path = api.beam_viterbi_2d(g[pre + 'log_trans'], g[pre + 'state_types'], g[pre + 'x'], g[pre + 'y'],
                                   g[pre + 'sub'], g[pre + 'pi'], env)
    ref = float(g[pre + 'viterbi_log_prob'])
    assert abs(lp - ref) <= 1e-12 * abs(ref)
    assert np.array_equal(np.asarray(path), g[pre + 'viterbi_path'])


@pytest.mark.parametrize('name', CASES)
def test_beam_sample_traceback_on_own_forward_table(cuda_lib, name):
    """Paths drawn on the GPU's pruned forward table with the reference's
    seed equal the reference's own draws on its float64 table (the tables
    agree to float32 rounding, far from any draw's cumulative-weight edge)."""
    from pairhmm import api
    g = load_golden('beam')
    pre = name + '_'
    args = _args(g, pre)
    lp, F, _ = api.beam_forward_2d(*args)
    rng = np.random.RandomState(int(g[pre + 'sample_seed']))
    lens = g[pre + 'sample_lens']
    rows = g[pre + 'sample_paths']
    ends = np.cumsum(lens)
    for a, b in zip(np.r_[0, ends[:-1]], ends):
        got = api.beam_sample_traceback(args[0], args[1], F, lp, args[2], args[3], args[4], args[5], rng, args[7])
        assert np.array_equal(np.asarray(got, np.int64).reshape(-1, 3), rows[a:b])
