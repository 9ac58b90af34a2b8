"""Stochastic forward traceback on the GPU (phmm_sample_paths) against the
float64 oracle (oracle/sample.py, the reference's sample_traceback_2d with
the product's counter-based stream): the same paths draw for draw, the
forward log-likelihood to 1e-12, and the sample frequencies of a small
lattice against its exact path probabilities."""
import numpy as np
import pytest

from test_sample_cpu import enumerate_paths, small_case

pytestmark = pytest.mark.gpu


def test_tiny_case_follows_posterior(cuda_lib):
    from pairhmm import api
    lt, st, emit, x, y, sub, pi = small_case()
    exact, ll_enum = enumerate_paths(lt, st, emit, len(x), len(y))
    n = 40000
    ll, paths = api.sample_traceback_2d_batch(lt, st, [x], [y], sub, pi, n, seed=2024)
    assert abs(ll[0] - ll_enum) <= 1e-12 * abs(ll_enum)
    freq = {}
    for pth in paths[0]:
        freq[tuple(pth)] = freq.get(tuple(pth), 0) + 1
    assert set(freq) <= set(exact)
    for k, p in exact.items():
        assert abs(freq.get(k, 0) / n - p) <= 5 * np.sqrt(p * (1 - p) / n) + 1e-9, (k, p)


@pytest.mark.parametrize('model', ['tkf91', 'mixdom'])
def test_paths_match_oracle(cuda_lib, model):
    from pairhmm import api, synth
    from pairhmm import models as pm
    from oracle import dp, sample, models as om
    rng = np.random.default_rng(81 if model == 'tkf91' else 82)
    Q, pi, _ = synth.rand_Q_pi(rng)
    t = 0.6
    if model == 'tkf91':
        lt = om.safe_log(om.tkf91_trans(0.03, 0.035, t))
        st = np.array([0, 1, 2, 3, 4], np.int8)
    else:
        p = synth.mixdom2_params(rng, 2, 1, 1)
        lt = om.safe_log(om.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'],
                                               p['dom_weights'], p['frag_weights'], p['ext_rates']))
        st = pm.mixdom_state_types(2, 1)
    sub = om.transition_matrix(Q, t)
    shapes = [(1, 1), (0, 4), (5, 0), (12, 17), (40, 33), (60, 71)]
    xs = [rng.integers(0, 20, a) for a, _ in shapes]
    ys = [rng.integers(0, 20, b) for _, b in shapes]
    S = 48
    ll, paths = api.sample_traceback_2d_batch(lt, st, xs, ys, sub, pi, S, seed=99)
    EM, EI, ED = dp.group_tables_tkf(sub, pi)
    for b in range(len(shapes)):
        emit = dp.log_emission_table(st, np.zeros(st.size, int), xs[b], ys[b], EM, EI, ED)
        ll_o, paths_o = sample.sample_paths(lt, st, emit, S, seed=99, pair=b)
        assert abs(ll[b] - ll_o) <= 1e-12 * abs(ll_o)
        assert len(paths[b]) == S
        same = sum(a == list(o) for a, o in zip(paths[b], paths_o))
        assert same == S, (b, same)


def test_single_path_api_and_zero_samples(cuda_lib):
    from pairhmm import api, _lib, synth
    from oracle import models as om
    rng = np.random.default_rng(5)
    Q, pi, _ = synth.rand_Q_pi(rng)
    lt = om.safe_log(om.tkf91_trans(0.03, 0.035, 0.5))
    st = np.array([0, 1, 2, 3, 4])
    x, y = rng.integers(0, 20, 9), rng.integers(0, 20, 11)
    sub = om.transition_matrix(Q, 0.5)
    lp, path = api.sample_traceback_2d(lt, st, x, y, sub, pi, np.array([0, 42], np.uint32))
    assert path[0] == (0, 0, 0) and path[-1][:2] == (9, 11)
    lp2, _ = api.viterbi_2d(lt, st, x, y, sub, pi)
    assert lp >= lp2   # forward log-likelihood >= best single path
    lM, lI, lD = api._log_tkf_tables(sub, pi)
    ll, p0 = _lib.sample_paths(st, np.zeros(5, np.int32), 1, [x], [y], lt[None], lM, lI, lD, 0, 1)
    assert p0 == [[]] and abs(ll[0] - lp) <= 1e-12 * abs(lp)
