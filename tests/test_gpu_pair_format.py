"""Pair records straight into the E-steps: the golden X/A/Y shard
(tests/golden/pairs.jsonl, written by the reference's encode_pair) read by
the native reader and run through the alignment-conditioned 1D E-step and
the match-aligned 2D E-step, against the float64 oracle on the reference's
own decode_pair outputs."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu


def _records():
    from pairhmm import pair_format as pf
    with open(os.path.join(GOLDEN, 'pairs.jsonl')) as f:
        return pf.read_records(f.read())


def test_records_into_1d_estep(cuda_lib):
    from pairhmm import api, synth
    from oracle import fb1d, models as om
    from pairhmm import models as pm
    g = load_golden('pairs')
    r = _records()
    rng = np.random.default_rng(17)
    K, F, C = 2, 1, 2
    p = synth.mixdom2_params(rng, K, F, C)
    cols, ancs, descs, ts = r.alignments()
    out = api.to_host(api.estep_1d_mixdom2(p, cols, ancs, descs, ts))
    st = pm.mixdom_state_types(K, F)
    for b in range(r.n_pairs):
        pre = f'p{b}_'
        t = float(g[pre + 't_est'])
        chi = om.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'], p['dom_weights'],
                                    p['frag_weights'], p['ext_rates'])
        csubs = om.build_class_subs(p['class_S_exch'], p['class_pis'], t)
        # the reference's decode_pair outputs expanded to columns
        states = g[pre + 'states']
        anc = np.full(states.size, 20)
        desc = np.full(states.size, 20)
        anc[states != 2] = g[pre + 'anc_chars']
        desc[states != 3] = g[pre + 'desc_chars']
        ll, _, n = fb1d.estep_1d(chi, st, states, anc, desc, csubs, p['class_pis'], p['classdist'], K, F)
        assert abs(out['log_p'][b] - ll) <= 1e-6 * abs(ll)
        np.testing.assert_allclose(out['n_trans'][b], n, rtol=1e-5, atol=1e-6)


def test_records_into_match_aligned_estep(cuda_lib):
    from pairhmm import api, synth
    from pairhmm import models as pm
    from oracle import dp, masked, models as om
    r = _records()
    rng = np.random.default_rng(19)
    K, F = 2, 1
    p = synth.mixdom2_params(rng, K, F, 1)
    t = 0.8
    lt = om.safe_log(om.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'],
                                           p['dom_weights'], p['frag_weights'], p['ext_rates']))
    st = pm.mixdom_state_types(K, F)
    subs, pis = [], []
    for _ in range(K):
        Q, pi, _ = synth.rand_Q_pi(rng)
        subs.append(om.transition_matrix(Q, t))
        pis.append(pi)
    subs, pis = np.stack(subs), np.stack(pis)
    xs, ys = r.sequences()
    mis, mjs = zip(*(r.match_positions(b) for b in range(r.n_pairs)))
    out = api.to_host(api.estep_batch_match_aligned(lt, st, xs, ys, mis, mjs, subs, pis, K, F))
    groups = np.zeros(st.size, np.int32)
    groups[2:] = np.arange(st.size - 2) // (5 * F)
    EM, EI, ED = dp.group_tables_per_domain(subs, pis, K)
    for b in range(r.n_pairs):
        emit = masked.mask_emissions_match_aligned(dp.log_emission_table(st, groups, xs[b], ys[b], EM, EI, ED),
                                                   st, mis[b], mjs[b])
        ll, post, n, _, _ = dp.forward_backward(lt, st, emit)
        assert abs(out['log_prob'][b] - ll) <= 1e-6 * abs(ll)
        np.testing.assert_allclose(out['expected_trans'][b], n, rtol=1e-5, atol=1e-6)
