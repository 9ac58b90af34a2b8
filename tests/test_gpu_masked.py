"""Cell-masked E-step on the GPU (phmm_batch.cell_mask, generic and two-warp
kernels) against the reference's own outputs (tests/golden/masked.npz) and
the float64 oracle (oracle/masked.py): the banded forward-backward around a
guide, forward_backward_2d on a match-aligned emission table, and the batched
match-aligned MixDom E-step.  Tolerances: log-likelihood 1e-6 relative,
counts 1e-5 relative (float32 DP against float64)."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu
BANDED = ('band_tkf91_a', 'band_tkf91_b', 'band_mixdom_a', 'band_tkf91_c')
MATCH = ('match_tkf91_a', 'match_mixdom_a', 'match_tkf91_b')


def _close_ll(a, b):
    assert abs(a - b) <= 1e-6 * abs(b), (a, b)


@pytest.mark.parametrize('name', BANDED)
def test_banded_matches_reference(cuda_lib, name):
    from pairhmm import api
    g = load_golden('masked')
    pre = name + '_'
    ll, post, n = api.forward_backward_2d_banded(g[pre + 'log_trans'], g[pre + 'state_types'], g[pre + 'x'],
                                                 g[pre + 'y'], g[pre + 'sub'], g[pre + 'pi'],
                                                 g[pre + 'band_center'], int(g[pre + 'band_width']))
    _close_ll(ll, float(g[pre + 'log_prob']))
    assert post.shape == g[pre + 'posteriors'].shape
    np.testing.assert_allclose(post, g[pre + 'posteriors'], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(n, g[pre + 'expected_trans'], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize('name', MATCH)
def test_match_aligned_table_matches_reference(cuda_lib, name):
    from pairhmm import api
    g = load_golden('masked')
    pre = name + '_'
    ll, post, n = api.forward_backward_2d(g[pre + 'log_trans'], g[pre + 'state_types'], g[pre + 'x'], g[pre + 'y'],
                                          None, None, log_emit_table=g[pre + 'log_emit'])
    _close_ll(ll, float(g[pre + 'log_prob']))
    gp = g[pre + 'posteriors']
    np.testing.assert_allclose(post, gp, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(n, g[pre + 'expected_trans'], rtol=1e-5, atol=1e-6)


def _rand_alignment(rng, Lx, Ly):
    n_m = int(rng.integers(min(Lx, Ly) // 2, min(Lx, Ly) + 1))
    states = np.array([1] * n_m + [3] * (Lx - n_m) + [2] * (Ly - n_m))
    rng.shuffle(states)
    xi = np.cumsum(np.isin(states, (1, 3))) - 1
    yj = np.cumsum(np.isin(states, (1, 2))) - 1
    return xi[states == 1], yj[states == 1]


@pytest.mark.parametrize('variant', [0, 1])
def test_match_aligned_batch_matches_oracle(cuda_lib, variant):
    """Batched match-aligned MixDom E-step (K=2 domains, F=1: 12 states; the
    automatic choice runs the two-warp kernels, variant 1 the generic ones)."""
    from pairhmm import api, synth
    from pairhmm import models as pm
    from oracle import dp, estep as oe, masked, models as om
    rng = np.random.default_rng(61 + variant)
    K, F = 2, 1
    p = synth.mixdom2_params(rng, K, F, 1)
    t = 0.5
    chi = om.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'], p['dom_weights'],
                                p['frag_weights'], p['ext_rates'])
    lt = om.safe_log(chi)
    st = pm.mixdom_state_types(K, F)
    subs, pis = [], []
    for _ in range(K):
        Q, pi, _ = synth.rand_Q_pi(rng)
        subs.append(om.transition_matrix(Q, t))
        pis.append(pi)
    subs, pis = np.stack(subs), np.stack(pis)
    shapes = [(1, 1), (7, 3), (40, 52), (95, 80), (150, 170)]
    xs = [rng.integers(0, 20, a) for a, _ in shapes]
    ys = [rng.integers(0, 20, b) for _, b in shapes]
    al = [_rand_alignment(rng, a, b) for a, b in shapes]
    groups = np.zeros(st.size, np.int32)
    groups[2:] = np.arange(st.size - 2) // (5 * F)
    plan = api.get_plan(st, groups, K)
    plan.set_variant(variant)
    try:
        r = api.estep_batch_match_aligned(lt, st, xs, ys, [a[0] for a in al], [a[1] for a in al], subs, pis, K, F)
        got = api.to_host(r)
        assert plan.last_variant == (7 if variant == 0 else variant)
    finally:
        plan.set_variant(0)
    EM, EI, ED = dp.group_tables_per_domain(subs, pis, K)
    for b in range(len(shapes)):
        emit = dp.log_emission_table(st, groups, xs[b], ys[b], EM, EI, ED)
        emit = masked.mask_emissions_match_aligned(emit, st, al[b][0], al[b][1])
        ll, post, n, _, _ = dp.forward_backward(lt, st, emit)
        _close_ll(got['log_prob'][b], ll)
        assert got['status'][b] == 0
        np.testing.assert_allclose(got['expected_trans'][b], n, rtol=1e-5, atol=1e-6)
        cM, cI, cD = oe.char_count_tables(post, st, groups, xs[b], ys[b], K)
        np.testing.assert_allclose(got['dom_match'][b], cM[:, :20, :20], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(got['dom_insert'][b], cI[:, :20], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(got['dom_delete'][b], cD[:, :20], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(got['agg_match'][b], cM[:, :20, :20].sum(axis=0), rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize('variant', [0, 1])
def test_band_mask_estep_matches_oracle(cuda_lib, variant):
    """Banded E-step over several stripes (TKF91, pairs up to 300 x 280, W = 10)
    through phmm_estep with a cell mask, against the oracle's banded model."""
    from pairhmm import api, synth, _lib
    from pairhmm import models as pm
    from oracle import dp, masked, models as om
    rng = np.random.default_rng(71 + variant)
    Q, pi, _ = synth.rand_Q_pi(rng)
    t = 0.4
    chi = om.tkf91_trans(0.03, 0.035, t)
    st = np.array([0, 1, 2, 3, 4], np.int8)
    sub = om.transition_matrix(Q, t)
    shapes = [(64, 70), (130, 129), (300, 280)]
    xs = [rng.integers(0, 20, a) for a, _ in shapes]
    ys = [rng.integers(0, 20, b) for _, b in shapes]
    centers = [np.round(np.arange(a + 1) * b / a).astype(int) for a, b in shapes]
    masks = [api.band_mask(a, b, c, 10) for (a, b), c in zip(shapes, centers)]
    EM, EI, ED = dp.group_tables_tkf(sub, pi)
    plan = api.get_plan(st, np.zeros(5, np.int32), 1)
    plan.set_variant(variant)
    try:
        bt = _lib.make_batch(xs, ys, chi[None], EM, EI, ED, cell_masks=masks)
        got = api.to_host(_lib.estep(plan, bt))
        assert plan.last_variant == (7 if variant == 0 else variant)
        ll_fwd, _ = _lib.forward(plan, bt)   # forward only, same kernels' forward
        ll_fwd = ll_fwd.cpu().numpy()
    finally:
        plan.set_variant(0)
    np.testing.assert_allclose(ll_fwd, got['ll'], rtol=1e-12)
    for b, (a, c) in enumerate(shapes):
        emit = dp.log_emission_table(st, np.zeros(5, int), xs[b], ys[b], EM, EI, ED)
        W = masked.pad_to_bin(10)
        emit[~masked.band_allowed(a, c, centers[b], W)] = om.NEG_INF
        ll, post, n, _, _ = dp.forward_backward(om.safe_log(chi), st, emit)
        _close_ll(got['ll'][b], ll)
        np.testing.assert_allclose(got['n_trans'][b], n, rtol=1e-5, atol=1e-6)


def test_band_excluding_origin_has_no_likelihood(cuda_lib):
    from pairhmm import api, synth, _lib
    from oracle import dp, models as om
    rng = np.random.default_rng(3)
    Q, pi, _ = synth.rand_Q_pi(rng)
    chi = om.tkf91_trans(0.03, 0.035, 0.4)
    st = np.array([0, 1, 2, 3, 4], np.int8)
    EM, EI, ED = dp.group_tables_tkf(om.transition_matrix(Q, 0.4), pi)
    x, y = rng.integers(0, 20, 20), rng.integers(0, 20, 30)
    mask = api.band_mask(20, 30, np.arange(21) + 10, 2)      # row 0 covers j = 8..12 only
    plan = api.get_plan(st, np.zeros(5, np.int32), 1)
    got = api.to_host(_lib.estep(plan, _lib.make_batch([x], [y], chi[None], EM, EI, ED, cell_masks=[mask])))
    assert got['ll'][0] <= -1e29
    assert got['status'][0] != 0
    assert np.all(got['n_trans'][0] == 0)


def test_mask_refused_by_other_families(cuda_lib):
    from pairhmm import api, synth, _lib
    from oracle import dp, models as om
    rng = np.random.default_rng(4)
    Q, pi, _ = synth.rand_Q_pi(rng)
    chi = om.tkf91_trans(0.03, 0.035, 0.4)
    st = np.array([0, 1, 2, 3, 4], np.int8)
    EM, EI, ED = dp.group_tables_tkf(om.transition_matrix(Q, 0.4), pi)
    x, y = rng.integers(0, 20, 20), rng.integers(0, 20, 30)
    mask = api.band_mask(20, 30, np.arange(21), 3)
    plan = api.get_plan(st, np.zeros(5, np.int32), 1)
    plan.set_variant(3)
    try:
        with pytest.raises(_lib.PairHMMError):
            _lib.estep(plan, _lib.make_batch([x], [y], chi[None], EM, EI, ED, cell_masks=[mask]))
    finally:
        plan.set_variant(0)


def test_band_layout_estep_multi_stripe_matches_oracle(cuda_lib):
    """phmm_estep_band (estep_batch_banded) over a batch of multi-stripe pairs
    (TKF91, up to 700 x 650, W = 16): the stripes skip the steps off their
    band, and the log-likelihoods, expected transitions and band-layout
    posteriors equal the oracle's banded model."""
    from pairhmm import api, synth
    from oracle import dp, masked, models as om
    rng = np.random.default_rng(91)
    Q, pi, _ = synth.rand_Q_pi(rng)
    t = 0.5
    chi = om.tkf91_trans(0.03, 0.035, t)
    st = np.array([0, 1, 2, 3, 4], np.int8)
    sub = om.transition_matrix(Q, t)
    shapes = [(700, 650), (200, 230), (64, 64), (65, 90)]
    xs = [rng.integers(0, 20, a) for a, _ in shapes]
    ys = [rng.integers(0, 20, b) for _, b in shapes]
    centers = [np.round(np.arange(a + 1) * b / a).astype(int) for a, b in shapes]
    ll, posts, n = api.estep_batch_banded(om.safe_log(chi), st, xs, ys, sub, pi, centers, 16)
    EM, EI, ED = dp.group_tables_tkf(sub, pi)
    W = masked.pad_to_bin(16)
    for b, (a, ly) in enumerate(shapes):
        emit = dp.log_emission_table(st, np.zeros(5, int), xs[b], ys[b], EM, EI, ED)
        emit[~masked.band_allowed(a, ly, centers[b], W)] = om.NEG_INF
        want_ll, post, want_n, _, _ = dp.forward_backward(om.safe_log(chi), st, emit)
        _close_ll(ll[b], want_ll)
        np.testing.assert_allclose(n[b], want_n, rtol=1e-5, atol=1e-6 * max(1.0, np.abs(want_n).max()))
        jj = centers[b][:, None] - W + np.arange(2 * W + 1)[None, :]
        ok = (jj >= 0) & (jj <= ly)
        want_pb = np.zeros((a + 1, 2 * W + 1, 5))
        ii, bb = np.nonzero(ok)
        want_pb[ii, bb] = post[ii, jj[ii, bb]]
        assert posts[b].shape[0] == masked.pad_to_bin(a) + 1
        np.testing.assert_allclose(posts[b][:a + 1], want_pb, rtol=1e-5, atol=1e-6)
        assert not posts[b][a + 1:].any()


def test_mask_with_an_empty_stripe(cuda_lib):
    """A mask that leaves no cell live in one 64-row stripe: that stripe and
    the ones below skip every step and wait on nothing; the pair has no
    likelihood and no counts, and the other pairs of the batch are exact."""
    from pairhmm import api, synth, _lib
    from oracle import dp, models as om
    rng = np.random.default_rng(5)
    Q, pi, _ = synth.rand_Q_pi(rng)
    chi = om.tkf91_trans(0.03, 0.035, 0.4)
    st = np.array([0, 1, 2, 3, 4], np.int8)
    EM, EI, ED = dp.group_tables_tkf(om.transition_matrix(Q, 0.4), pi)
    shapes = [(200, 190), (150, 160)]
    xs = [rng.integers(0, 20, a) for a, _ in shapes]
    ys = [rng.integers(0, 20, b) for _, b in shapes]
    masks = [api.band_mask(a, b, np.round(np.arange(a + 1) * b / a).astype(int), 12) for a, b in shapes]
    masks[0][64:128] = 0
    plan = api.get_plan(st, np.zeros(5, np.int32), 1)
    got = api.to_host(_lib.estep(plan, _lib.make_batch(xs, ys, chi[None], EM, EI, ED, cell_masks=masks)))
    assert plan.last_variant == 7
    assert got['ll'][0] <= -1e29 and got['status'][0] != 0 and not got['n_trans'][0].any()
    emit = dp.log_emission_table(st, np.zeros(5, int), xs[1], ys[1], EM, EI, ED)
    emit[masks[1] == 0] = om.NEG_INF
    ll, _, n, _, _ = dp.forward_backward(om.safe_log(chi), st, emit)
    assert got['status'][1] == 0
    _close_ll(got['ll'][1], ll)
    np.testing.assert_allclose(got['n_trans'][1], n, rtol=1e-5, atol=1e-6)
