"""2D Viterbi on the GPU (phmm_viterbi) against the reference's outputs
(tests/golden/viterbi.npz) and the float64 oracle: the same best path and
log-probability (float64 on both sides: 1e-12 relative)."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu
CASES = ('tkf91_a', 'tkf91_b', 'tkf91_e', 'mixdom_a')


@pytest.mark.parametrize('name', CASES)
def test_matches_reference(cuda_lib, name):
    from pairhmm import api
    g = load_golden('viterbi')
    pre = name + '_'
    lp, path = api.viterbi_2d(g[pre + 'log_trans'], g[pre + 'state_types'], g[pre + 'x'], g[pre + 'y'],
                              g[pre + 'sub'], g[pre + 'pi'])
    assert abs(lp - g[pre + 'log_prob']) <= 1e-12 * abs(g[pre + 'log_prob'])
    assert np.array_equal(np.asarray(path), g[pre + 'path'])


def test_ragged_batch_matches_oracle(cuda_lib):
    from pairhmm import api, synth
    from pairhmm import models as pm
    from oracle import viterbi, models as om
    rng = np.random.default_rng(95)
    K, F = 3, 1
    p = synth.mixdom2_params(rng, K, F, 1)
    Q, pi, _ = synth.rand_Q_pi(rng)
    t = 0.6
    chi = om.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'], p['dom_weights'],
                                p['frag_weights'], p['ext_rates'])
    lt = om.safe_log(chi)
    st = pm.mixdom_state_types(K, F)
    sub = om.transition_matrix(Q, t)
    shapes = [(1, 1), (1, 9), (12, 1), (30, 33), (64, 70), (120, 95)]
    xs = [rng.integers(0, 20, a) for a, _ in shapes]
    ys = [rng.integers(0, 20, b) for _, b in shapes]
    ll, paths = api.viterbi_2d_batch(lt, st, xs, ys, sub, pi)
    for b in range(len(shapes)):
        want_lp, want_path = viterbi.viterbi_2d(lt, st, xs[b], ys[b], sub, pi)
        assert abs(ll[b] - want_lp) <= 1e-12 * abs(want_lp), b
        assert paths[b] == [tuple(v) for v in want_path], b
