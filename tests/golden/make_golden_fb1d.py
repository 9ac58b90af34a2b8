"""Golden fixtures for the 1D alignment-conditioned forward-backward, produced
by the reference's own modules: ``dp/hmm.py`` ``forward_backward_1d_padded``
(sequential and associative scans) on emission tables from
``pair_hmm_emissions_constrained_per_class`` (MixDom2, per-class mixture) and
``pair_hmm_emissions_constrained_per_domain`` (MixDom1), with chi from
``models/mixdom.py`` ``build_nested_trans``.

Usage (needs the reference checkout; writes tests/golden/fb1d.npz):

    python tests/golden/make_golden_fb1d.py <reference>/python

JAX is replaced by the NumPy stand-in of ``jax_shim.py``.  Alignments are
seeded random column-type strings (M / I / D) with random characters.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import jax_shim  # noqa: E402
from make_golden import rand_mixdom2  # noqa: E402


def main(ref_python):
    jax_shim.install()
    sys.path.insert(0, ref_python)
    from tkfmixdom.jax.dp import hmm
    from tkfmixdom.jax.models import mixdom
    from tkfmixdom.jax.core import ctmc
    rng = np.random.default_rng(20261205)
    out = {}
    cases = (('k2f1c2', 2, 1, 2, 23, 30), ('k3f1c1', 3, 1, 1, 17, 25), ('k2f2c3', 2, 2, 3, 11, 40),
             ('k1f1c1_short', 1, 1, 1, 1, 4))
    for name, K, F, C, L, Lpad in cases:
        p = rand_mixdom2(rng, K, F, C, False)
        t = float(np.exp(rng.uniform(np.log(0.1), np.log(1.5))))
        chi, _ = mixdom.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'],
                                           p['dom_weights'], p['frag_weights'], p['ext_rates'])
        chi = np.asarray(chi)
        st = np.asarray(mixdom.state_types(K, F))
        Q = [np.asarray(p['class_S_exch'][c]) * p['class_pis'][c][None, :] for c in range(C)]
        for q in Q:
            np.fill_diagonal(q, 0.0)
            np.fill_diagonal(q, -q.sum(axis=1))
        csubs = np.stack([np.asarray(ctmc.transition_matrix(q, t)) for q in Q])
        cols = rng.choice(np.array([1, 2, 3]), size=L, p=[0.6, 0.2, 0.2]).astype(np.int32)
        anc = rng.integers(0, 20, L).astype(np.int32)
        desc = rng.integers(0, 20, L).astype(np.int32)
        if L > 4:
            anc[2] = 20
            desc[3] = 20
        emit = np.asarray(hmm.pair_hmm_emissions_constrained_per_class(
            st, cols, anc, desc, csubs, p['class_pis'], p['classdist'], K, F))
        lt = jax_shim._wrap(np.asarray(hmm.safe_log(chi)))
        emit_pad = np.full((Lpad, emit.shape[1]), -1e30)
        emit_pad[:L] = emit
        emit_pad = jax_shim._wrap(emit_pad)
        e_idx = int(hmm._find_e_idx(st))   # MixDom's End state (index 1), as the callers pass it
        lp_s, post_s, nt_s = hmm.forward_backward_1d_padded(lt, emit_pad, L, init_state=0, final_state=e_idx,
                                                            scan_mode='sequential')
        lp_a, post_a, nt_a = hmm.forward_backward_1d_padded(lt, emit_pad, L, init_state=0, final_state=e_idx)
        if L > 1:   # (the stand-in's scan cannot stack an empty sequence of steps)
            lp_p, post_p, nt_p = hmm.forward_backward_1d(lt, jax_shim._wrap(emit), init_state=0,
                                                         final_state=e_idx)
        else:
            lp_p, nt_p = lp_s, nt_s
        pre = name + '_'
        for k in ('main_ins', 'main_del', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates',
                  'class_pis', 'class_S_exch', 'classdist'):
            out[pre + 'p_' + k] = np.asarray(p[k], dtype=np.float64)
        out[pre + 't'] = np.float64(t)
        out[pre + 'chi'] = chi
        out[pre + 'state_types'] = st
        out[pre + 'csubs'] = csubs
        out[pre + 'cols'] = cols
        out[pre + 'anc'] = anc
        out[pre + 'desc'] = desc
        out[pre + 'log_emit'] = emit
        out[pre + 'log_prob'] = np.float64(lp_s)
        out[pre + 'posteriors'] = np.asarray(post_s)
        out[pre + 'expected_trans'] = np.asarray(nt_s)
        out[pre + 'log_prob_assoc'] = np.float64(lp_a)
        out[pre + 'expected_trans_assoc'] = np.asarray(nt_a)
        out[pre + 'log_prob_plain'] = np.float64(lp_p)
        out[pre + 'expected_trans_plain'] = np.asarray(nt_p)
        out[pre + 'Lpad'] = np.int64(Lpad)
        out[pre + 'e_idx'] = np.int64(e_idx)
    path = os.path.join(HERE, 'fb1d.npz')
    np.savez_compressed(path, **out)
    print('wrote', path, len(out), 'arrays')


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden_fb1d.py <reference checkout>/python')
    main(sys.argv[1])
