"""The C half of the oracle (oracle/fb2d.c) against the NumPy oracle
(oracle/dp.py, itself pinned to the reference's outputs): log-likelihood and
expected transitions on TKF91, MixDom2 and 42-state models, empty sequences
and the golden fixtures' pairs."""
import numpy as np
import pytest

from conftest import load_golden


@pytest.fixture(scope='module')
def cdp():
    from oracle import build_oracle, cdp
    build_oracle.build()
    return cdp


def _model(rng, kind):
    from oracle import dp, models as om, estep as oe
    from pairhmm import synth
    if kind == 'tkf91':
        Q, pi, _ = synth.rand_Q_pi(rng)
        chi = om.tkf91_trans(0.03, 0.035, 0.7)
        EM, EI, ED = dp.group_tables_tkf(om.transition_matrix(Q, 0.7), pi)
        return chi, np.array([0, 1, 2, 3, 4]), np.zeros(5, int), EM, EI, ED
    K, F, C = (3, 1, 1) if kind == 'mixdom17' else (4, 2, 2)
    p = synth.mixdom2_params(rng, K, F, C)
    p['t'] = 0.5
    chi, st, groups, EM, EI, ED, _ = oe.mixdom2_model(p)
    return chi, st, groups, EM, EI, ED


@pytest.mark.parametrize('kind', ['tkf91', 'mixdom17', 'mixdom42'])
def test_c_oracle_matches_numpy(cdp, kind):
    from oracle import dp, models as om
    rng = np.random.default_rng({'tkf91': 1, 'mixdom17': 2, 'mixdom42': 3}[kind])
    chi, st, groups, EM, EI, ED = _model(rng, kind)
    lt = om.safe_log(chi)
    for Lx, Ly in ((0, 0), (0, 5), (4, 0), (1, 1), (13, 9), (30, 41)):
        x, y = rng.integers(0, 21, Lx), rng.integers(0, 21, Ly)
        emit = dp.log_emission_table(st, groups, x, y, EM, EI, ED)
        ll, _, n, _, _ = dp.forward_backward(lt, st, emit)
        ll_c, n_c = cdp.forward_backward(lt, st, emit)
        assert abs(ll_c - ll) <= 1e-12 * max(1.0, abs(ll))
        np.testing.assert_allclose(n_c, n, rtol=1e-10, atol=1e-12)
        llf, nf = cdp.forward_backward(lt, st, emit, forward_only=True)
        assert llf == ll_c and nf is None


@pytest.mark.parametrize('name', ['tkf91', 'tkf92', 'mixdom2_k3f1c1'])
def test_c_oracle_on_golden_pairs(cdp, name):
    """The fixtures' own pairs through the C oracle give the reference's
    log-likelihood and expected transitions."""
    from oracle import dp, models as om
    g = load_golden(name)
    lt = om.safe_log(g['chi'])
    if name.startswith('tkf'):
        st = np.array([0, 1, 2, 3, 4])
        EM, EI, ED = dp.group_tables_tkf(g['sub'], g['p_pi'])
        emit = dp.log_emission_table(st, np.zeros(5, int), g['x'], g['y'], EM, EI, ED)
        ll_ref, n_ref = float(g['ll_fb']), g['n_trans']
    else:
        st = om.mixdom_state_types(int(g['K']), int(g['F']))
        emit = g['log_emit'][:len(g['x']) + 1, :len(g['y']) + 1]
        ll_ref, n_ref = float(g['ll']), g['n_trans']
    ll_c, n_c = cdp.forward_backward(lt, st, emit)
    assert abs(ll_c - ll_ref) <= 1e-10 * abs(ll_ref)
    np.testing.assert_allclose(n_c, n_ref, rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize('kind', ['tkf91', 'mixdom17', 'mixdom42'])
def test_c_oracle_char_counts_match_numpy(cdp, kind):
    from oracle import dp, models as om, estep as oe
    rng = np.random.default_rng({'tkf91': 4, 'mixdom17': 5, 'mixdom42': 6}[kind])
    chi, st, groups, EM, EI, ED = _model(rng, kind)
    lt = om.safe_log(chi)
    G = int(np.max(groups)) + 1
    for Lx, Ly in ((0, 3), (2, 0), (9, 12), (25, 21)):
        x, y = rng.integers(0, 21, Lx), rng.integers(0, 21, Ly)
        emit = dp.log_emission_table(st, groups, x, y, EM, EI, ED)
        ll, post, n, _, _ = dp.forward_backward(lt, st, emit)
        want = oe.char_count_tables(post, st, groups, x, y, G)
        _, _, got = cdp.forward_backward(lt, st, emit, counts=(groups, G, x, y))
        for a, b in zip(got, want):
            np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize('kind', ['tkf91', 'mixdom17'])
def test_tiny_lattices_exhaustively(cdp, kind):
    """Every Lx, Ly in 0..4 (the edge cases of empty, single-residue and
    narrow lattices): both halves of the oracle agree on the likelihood,
    the expected transitions and the character counts."""
    from oracle import dp, models as om, estep as oe
    rng = np.random.default_rng(7 if kind == 'tkf91' else 8)
    chi, st, groups, EM, EI, ED = _model(rng, kind)
    lt = om.safe_log(chi)
    G = int(np.max(groups)) + 1
    for Lx in range(5):
        for Ly in range(5):
            x, y = rng.integers(0, 21, Lx), rng.integers(0, 21, Ly)
            emit = dp.log_emission_table(st, groups, x, y, EM, EI, ED)
            ll, post, n, _, _ = dp.forward_backward(lt, st, emit)
            ll_c, n_c, cnt = cdp.forward_backward(lt, st, emit, counts=(groups, G, x, y))
            assert abs(ll_c - ll) <= 1e-12 * max(1.0, abs(ll)), (Lx, Ly)
            np.testing.assert_allclose(n_c, n, rtol=1e-10, atol=1e-12)
            for a, b in zip(cnt, oe.char_count_tables(post, st, groups, x, y, G)):
                np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-12)
