"""Host-side helpers of the masked, banded and beam paths on the CPU: the
cell masks, the band layout, the envelope builder against the oracle's
restatement of the reference, the refinement's envelope dilation, masked
emission-table decomposition, the seed of a PRNG key and the output arena."""
import numpy as np
import pytest
import torch


def _rand_guide(rng, Lx, Ly):
    n_m = int(rng.integers(0, min(Lx, Ly) + 1))
    states = np.array([1] * n_m + [3] * (Lx - n_m) + [2] * (Ly - n_m))
    rng.shuffle(states)
    mx = np.where(np.isin(states, (1, 3)), 0, -1)
    my = np.where(np.isin(states, (1, 2)), 0, -1)
    return mx, my


@pytest.mark.parametrize('seed', range(6))
def test_envelope_matches_oracle(seed):
    from pairhmm import api
    from oracle import beam
    rng = np.random.default_rng(seed)
    Lx, Ly = (int(v) for v in rng.integers(0, 40, 2))
    mx, my = _rand_guide(rng, Lx, Ly)
    bw = int(rng.integers(0, 6))
    assert np.array_equal(api.msa_to_envelope(Lx, Ly, mx, my, bw), beam.msa_to_envelope(Lx, Ly, mx, my, bw))


def test_band_mask_and_layout():
    from pairhmm import api
    from oracle import masked
    rng = np.random.default_rng(1)
    Lx, Ly, bw = 17, 23, 2
    c = np.clip(np.round(np.arange(Lx + 1) * Ly / Lx).astype(int) + rng.integers(-2, 3, Lx + 1), 0, Ly)
    m = api.band_mask(Lx, Ly, c, bw)
    W = masked.pad_to_bin(bw)
    assert np.array_equal(m == 7, masked.band_allowed(Lx, Ly, c, W))
    assert set(np.unique(m)) <= {0, 7}
    dense = rng.random((Lx + 1, Ly + 1, 5))
    assert np.array_equal(api._to_band_layout(dense, c, W), masked.to_band_layout(dense, c, W))


def test_match_aligned_mask_bits():
    from pairhmm import api
    m = api.match_aligned_mask(4, 5, [0, 2, 3], [1, 2, 4])
    assert m.shape == (5, 6)
    assert set(zip(*np.nonzero(m & 1))) == {(1, 2), (3, 3), (4, 5)}
    assert np.all(m & 6 == 6)


def test_masked_table_decomposition():
    """forward_backward_2d's table path recovers the character tables and the
    type mask of a match-aligned table, and refuses a table whose entries do
    not depend on the characters alone."""
    from pairhmm import api
    from oracle import dp, masked
    rng = np.random.default_rng(2)
    st = np.array([0, 1, 2, 3, 4])
    pi = rng.dirichlet(np.ones(20))
    sub = rng.dirichlet(np.ones(20), size=20)
    EM, EI, ED = dp.group_tables_tkf(sub, pi)
    x, y = rng.integers(0, 20, 9), rng.integers(0, 20, 7)
    emit = dp.log_emission_table(st, np.zeros(5, int), x, y, EM, EI, ED)
    groups, TM, TI, TD, mask = api._groups_from_table(emit, st, x, y)
    assert mask is None
    mi, mj = np.array([0, 3, 5]), np.array([1, 2, 6])
    le = masked.mask_emissions_match_aligned(emit, st, mi, mj)
    groups, TM, TI, TD, mask = api._groups_from_table(le, st, x, y)
    want = api.match_aligned_mask(9, 7, mi, mj)
    want[0, :] |= 5
    want[:, 0] |= 3
    assert np.array_equal(mask, want)
    bad = emit.copy()
    bad[2, 3, 2] += 0.5
    with pytest.raises(NotImplementedError):
        api._groups_from_table(bad, st, x, y)


def test_refinement_dilation_matches_box_union():
    """The difference-array dilation of iterative_beam_refinement equals the
    reference's union of clipped boxes around the active cells."""
    rng = np.random.default_rng(3)
    Lx, Ly, nb = 20, 25, 3
    active = rng.random((Lx + 1, Ly + 1)) < 0.05
    want = np.zeros_like(active)
    for i, j in zip(*np.nonzero(active)):
        want[max(0, i - nb):min(Lx, i + nb) + 1, max(0, j - nb):min(Ly, j + nb) + 1] = True
    ii, jj = np.nonzero(active)
    acc = np.zeros((Lx + 2, Ly + 2), np.int64)
    np.add.at(acc, (np.maximum(ii - nb, 0), np.maximum(jj - nb, 0)), 1)
    np.add.at(acc, (np.minimum(ii + nb, Lx) + 1, np.maximum(jj - nb, 0)), -1)
    np.add.at(acc, (np.maximum(ii - nb, 0), np.minimum(jj + nb, Ly) + 1), -1)
    np.add.at(acc, (np.minimum(ii + nb, Lx) + 1, np.minimum(jj + nb, Ly) + 1), 1)
    got = acc.cumsum(axis=0).cumsum(axis=1)[:Lx + 1, :Ly + 1] > 0
    assert np.array_equal(got, want)


def test_seed_of_prng_keys():
    from pairhmm import api
    assert api._seed_of(5) == 5
    assert api._seed_of(-1) == (1 << 64) - 1
    assert api._seed_of(np.array([0, 42], np.uint32)) == 42 << 32
    assert api._seed_of(np.array([7, 1], np.uint32)) == 7 | (1 << 32)


def test_output_arena_and_host_copy_on_cpu():
    from pairhmm import _lib
    ar = _lib.OutputArena('cpu', [('a', (3, 4), torch.float64), ('b', (5,), torch.int32),
                                  ('c', (2, 2, 2), torch.float64)])
    for name, shape in (('a', (3, 4)), ('b', (5,)), ('c', (2, 2, 2))):
        assert tuple(ar[name].shape) == shape
        assert (ar[name].data_ptr() - ar.buf.data_ptr()) % 256 == 0   # slices 256-byte aligned in the buffer
    assert ar['a'].untyped_storage().data_ptr() == ar['c'].untyped_storage().data_ptr()
    ar['a'].fill_(1.5)
    ar['b'].fill_(7)
    host = _lib.to_host({'a': ar['a'], 'b': ar['b'], 'note': 'kept'})
    assert np.all(host['a'] == 1.5) and np.all(host['b'] == 7) and host['note'] == 'kept'


@pytest.mark.parametrize('name', ['band_tkf91_a', 'band_tkf91_b', 'band_mixdom_a', 'band_tkf91_c', 'band_tkf91_d'])
def test_msa_to_band_center_matches_reference(name):
    from conftest import load_golden
    from pairhmm import api
    g = load_golden('masked')
    pre = name + '_'
    bc = api.msa_to_band_center(g[pre + 'msa_x'], g[pre + 'msa_y'], len(g[pre + 'x']))
    assert bc.dtype == np.int32 and np.array_equal(bc, g[pre + 'band_center'])


@pytest.mark.parametrize('name', ['match_tkf91_a', 'match_mixdom_a', 'match_tkf91_b'])
def test_mask_emissions_match_aligned_matches_reference(name):
    from conftest import load_golden
    from pairhmm import api
    from oracle import dp
    g = load_golden('masked')
    pre = name + '_'
    st = g[pre + 'state_types']
    EM, EI, ED = dp.group_tables_tkf(g[pre + 'sub'], g[pre + 'pi'])
    emit = dp.log_emission_table(st, np.zeros(st.size, int), g[pre + 'x'], g[pre + 'y'], EM, EI, ED)
    got = api.mask_emissions_match_aligned(emit, st, g[pre + 'match_i'], g[pre + 'match_j'])
    ref = g[pre + 'log_emit']
    assert np.array_equal(got > -1e29, ref > -1e29)
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize('name', ['mixdom2_k3f1c1', 'mixdom2_k2f2c2', 'mixdom2_k1f2c3_wild', 'mixdom1_d3f2'])
def test_dense_emission_builders_match_reference(name):
    """pair_hmm_emissions_per_class / _per_domain against the reference's own
    tables in the MixDom fixtures (wildcards included)."""
    from conftest import load_golden
    from pairhmm import api
    from pairhmm import models as pm
    g = load_golden(name)
    K, F = int(g['K']), int(g['F'])
    st = pm.mixdom_state_types(K, F)
    if name.startswith('mixdom2'):
        got = api.pair_hmm_emissions_per_class(st, g['x'], g['y'], g['class_subs'], g['p_class_pis'],
                                               g['p_classdist'], K, F)
    else:
        got = api.pair_hmm_emissions_per_domain(st, g['x'], g['y'], g['subs'], g['dom_pis'], K, F)
    ref = g['log_emit'][:len(g['x']) + 1, :len(g['y']) + 1]
    live = ref > -1e29
    assert np.array_equal(live, got > -1e29)
    np.testing.assert_allclose(got[live], ref[live], rtol=1e-12, atol=1e-12)


def test_pair_hmm_emissions_matches_oracle():
    from pairhmm import api
    from oracle import dp
    rng = np.random.default_rng(8)
    pi = rng.dirichlet(np.ones(20))
    sub = rng.dirichlet(np.ones(20), size=20)
    st = np.array([0, 1, 2, 3, 4])
    x, y = rng.integers(0, 21, 11), rng.integers(0, 21, 7)
    EM, EI, ED = dp.group_tables_tkf(sub, pi)
    want = dp.log_emission_table(st, np.zeros(5, int), x, y, EM, EI, ED)
    got = api.pair_hmm_emissions(st, x, y, sub, pi)
    emitting = np.isin(st, (1, 2, 3))
    np.testing.assert_allclose(got[:, :, emitting], want[:, :, emitting], rtol=1e-13, atol=1e-13)
    assert np.all(got[:, :, ~emitting] == 0.0)
