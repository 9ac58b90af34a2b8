"""Golden fixtures for the 2D Viterbi decoder, produced by the reference's own
``dp/hmm.py`` ``viterbi_2d`` (TKF91 and a MixDom model with one substitution
model, chi from ``models/mixdom.py`` ``build_nested_trans``).

Usage (needs the reference checkout; writes tests/golden/viterbi.npz):

    python tests/golden/make_golden_viterbi.py <reference>/python

JAX is replaced by the NumPy stand-in of ``jax_shim.py``; the sequences hold
no wildcard (the reference's viterbi_2d indexes a 20 x 20 matrix).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import jax_shim  # noqa: E402
from make_golden import rand_Q_pi, rand_mixdom2  # noqa: E402


def main(ref_python):
    jax_shim.install()
    sys.path.insert(0, ref_python)
    from tkfmixdom.jax.dp import hmm
    from tkfmixdom.jax.models import mixdom
    from tkfmixdom.jax.core import params as cp, ctmc
    rng = np.random.default_rng(20261206)
    out = {}
    cases = (('tkf91_a', 'tkf91', 6, 7), ('tkf91_b', 'tkf91', 9, 4), ('tkf91_e', 'tkf91', 1, 3),
             ('mixdom_a', 'mixdom', 7, 8))
    for name, model, Lx, Ly in cases:
        Q, pi, _ = rand_Q_pi(rng)
        t = float(np.exp(rng.uniform(np.log(0.2), np.log(1.2))))
        if model == 'tkf91':
            lam = rng.uniform(0.01, 0.05)
            chi = np.asarray(cp.tkf91_trans(lam, lam * rng.uniform(1.05, 1.5), t))
            st = np.array([0, 1, 2, 3, 4])
        else:
            p = rand_mixdom2(rng, 2, 1, 1, False)
            chi = np.asarray(mixdom.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'],
                                                       p['dom_weights'], p['frag_weights'], p['ext_rates'])[0])
            st = np.asarray(mixdom.state_types(2, 1))
        sub = np.asarray(ctmc.transition_matrix(Q, t))
        x = rng.integers(0, 20, Lx).astype(np.int32)
        y = rng.integers(0, 20, Ly).astype(np.int32)
        lt = jax_shim._wrap(np.asarray(hmm.safe_log(chi)))
        lp, path = hmm.viterbi_2d(lt, jax_shim._wrap(st), jax_shim._wrap(x), jax_shim._wrap(y),
                                  jax_shim._wrap(sub), jax_shim._wrap(pi))
        pre = name + '_'
        out[pre + 'log_trans'] = np.asarray(lt)
        out[pre + 'state_types'] = st
        out[pre + 'x'] = x
        out[pre + 'y'] = y
        out[pre + 'sub'] = sub
        out[pre + 'pi'] = pi
        out[pre + 'log_prob'] = np.float64(lp)
        out[pre + 'path'] = np.asarray(path, np.int64).reshape(-1, 3)
    path = os.path.join(HERE, 'viterbi.npz')
    np.savez_compressed(path, **out)
    print('wrote', path, len(out), 'arrays')


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden_viterbi.py <reference checkout>/python')
    main(sys.argv[1])
