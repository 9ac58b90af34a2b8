"""Golden fixtures for the exact MixDom sufficient statistics, produced by the
reference's own modules (``models/exact_suffstats.py`` per pair and
``models/exact_suffstats_batch.py`` batched; they build the fully exploded
model of ``models/fully_exploded.py`` and walk the elimination chain of
``models/elimination_steps.py``).

Usage (needs the reference checkout; writes tests/golden/exact_suffstats.npz):

    python tests/golden/make_golden_suffstats.py <reference>/python

JAX is replaced by the NumPy stand-in of ``jax_shim.py``.  The collapsed
counts n_chi are seeded random non-negative matrices on the support of chi
(the restoration is linear in n_chi, so any counts exercise it); every
output array is a reference output, stored beside its inputs.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import jax_shim  # noqa: E402
from make_golden import rand_mixdom2  # noqa: E402

KEYS = ('top_5x5', 'dom_M_5x5', 'dom_kappa', 'dom_1mkappa', 'ext', 'term', 'dom_w', 'frag_w')


def main(ref_python):
    jax_shim.install()
    sys.path.insert(0, ref_python)
    from tkfmixdom.jax.models import mixdom, exact_suffstats as es, exact_suffstats_batch as esb
    rng = np.random.default_rng(20261204)
    out = {}
    cases = (('k2f1', 2, 1, False, False), ('k3f2', 3, 2, False, False), ('k2f2x', 2, 2, True, False),
             ('k2f1eq', 2, 1, False, True))
    for name, K, F, ext_full, equal in cases:
        p = rand_mixdom2(rng, K, F, 1, ext_full)
        if equal:   # lambda ~ mu at the domain level (the L'Hopital branches)
            p['dom_del'] = p['dom_ins'] * (1 + 2e-5)
        B = 3
        ts = np.exp(rng.uniform(np.log(0.05), np.log(2.0), B))
        N = 2 + 5 * K * F
        n_stack = []
        per_pair = {k: [] for k in KEYS}
        for b in range(B):
            chi = np.asarray(mixdom.build_nested_trans(
                p['main_ins'], p['main_del'], ts[b], p['dom_ins'], p['dom_del'], p['dom_weights'],
                p['frag_weights'], p['ext_rates'])[0])
            n = rng.gamma(1.0, 2.0, (N, N)) * (chi > 0)
            n_stack.append(n)
            ss = es.exact_suffstats(n, p['main_ins'], p['main_del'], ts[b], p['dom_ins'], p['dom_del'],
                                    p['dom_weights'], p['frag_weights'], p['ext_rates'])
            for k in KEYS:
                per_pair[k].append(np.asarray(ss[k]))
        n_stack = np.stack(n_stack)
        bs = esb.exact_suffstats_batch(n_stack, p['main_ins'], p['main_del'], ts, p['dom_ins'], p['dom_del'],
                                       p['dom_weights'], p['frag_weights'], p['ext_rates'])
        pre = name + '_'
        for k in ('main_ins', 'main_del', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates'):
            out[pre + 'p_' + k] = np.asarray(p[k], dtype=np.float64)
        out[pre + 't'] = ts
        out[pre + 'n_chi'] = n_stack
        for k in KEYS:
            out[pre + 'ss_' + k] = np.stack(per_pair[k])              # per-pair reference
            v = bs[k]
            out[pre + 'bs_' + k] = np.stack(v, axis=1) if isinstance(v, list) else np.asarray(v)
    path = os.path.join(HERE, 'exact_suffstats.npz')
    np.savez_compressed(path, **out)
    print('wrote', path, len(out), 'arrays')


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden_suffstats.py <reference checkout>/python')
    main(sys.argv[1])
