"""Golden fixtures for the masked 2D forward-backward variants, produced by the
reference's own ``dp/hmm.py``: ``forward_backward_2d_banded`` around an MSA
guide (band centres from ``msa_to_band_center``) and ``forward_backward_2d`` on
an emission table masked by ``mask_emissions_match_aligned`` (the match-aligned
training E-step of train_pfam.py), for TKF91 and a MixDom model with one
substitution model (chi from ``models/mixdom.py`` ``build_nested_trans``).

Usage (needs the reference checkout; writes tests/golden/masked.npz):

    python tests/golden/make_golden_masked.py <reference>/python

JAX is replaced by the NumPy stand-in of ``jax_shim.py``.  Guide alignments
are seeded random M/I/D strings of the pair's lengths.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import jax_shim  # noqa: E402
from make_golden import rand_Q_pi, rand_mixdom2  # noqa: E402


def rand_alignment(rng, Lx, Ly):
    """M/I/D states (1/2/3) with Lx M+D and Ly M+I columns, and the MSA rows."""
    n_m = int(rng.integers(max(0, min(Lx, Ly) // 2), min(Lx, Ly) + 1))
    states = np.array([1] * n_m + [3] * (Lx - n_m) + [2] * (Ly - n_m))
    rng.shuffle(states)
    mx, my = [], []
    xi = yj = 0
    for s in states:
        mx.append(xi if s in (1, 3) else -1)
        my.append(yj if s in (1, 2) else -1)
        xi += s in (1, 3)
        yj += s in (1, 2)
    return states, np.array(mx), np.array(my)


def main(ref_python):
    jax_shim.install()
    sys.path.insert(0, ref_python)
    from tkfmixdom.jax.dp import hmm
    from tkfmixdom.jax.models import mixdom
    from tkfmixdom.jax.core import params as cp, ctmc
    rng = np.random.default_rng(20261207)
    w = jax_shim._wrap
    out = {}
    # Lx at a padding bin (17, 30, 14, 8) except band_tkf91_d: the reference's
    # banded backward starts from the terminal band placed at row pad_to_bin(Lx)
    # (dp/hmm.py:2337-2343), so its posteriors and counts are those of the
    # banded model only when Lx is a bin size; band_tkf91_d records that case
    cases = (('band_tkf91_a', 'band', 'tkf91', 17, 22, 2), ('band_tkf91_b', 'band', 'tkf91', 30, 26, 5),
             ('band_mixdom_a', 'band', 'mixdom', 14, 17, 3), ('band_tkf91_c', 'band', 'tkf91', 8, 3, 1),
             ('band_tkf91_d', 'band', 'tkf91', 18, 22, 2),
             ('match_tkf91_a', 'match', 'tkf91', 15, 19, 0), ('match_mixdom_a', 'match', 'mixdom', 12, 14, 0),
             ('match_tkf91_b', 'match', 'tkf91', 6, 2, 0))
    for name, kind, model, Lx, Ly, bw in cases:
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
        states, mx, my = rand_alignment(rng, Lx, Ly)
        lt = w(np.asarray(hmm.safe_log(chi)))
        pre = name + '_'
        if kind == 'band':
            bc = np.asarray(hmm.msa_to_band_center(mx, my, Lx))
            lp, post, nt = hmm.forward_backward_2d_banded(lt, w(st), w(x), w(y), w(sub), w(pi), w(bc), bw)
            out[pre + 'band_center'] = bc
            out[pre + 'band_width'] = np.int64(bw)
            out[pre + 'msa_x'] = mx
            out[pre + 'msa_y'] = my
        else:
            mi = np.array([mx[c] for c in range(len(states)) if states[c] == 1], np.int32)
            mj = np.array([my[c] for c in range(len(states)) if states[c] == 1], np.int32)
            emit = hmm.pair_hmm_emissions(w(st), w(x), w(y), w(sub), w(pi))
            masked = hmm.mask_emissions_match_aligned(emit, w(st), w(mi), w(mj))
            lp, post, nt = hmm.forward_backward_2d(lt, w(st), w(x), w(y), w(sub), w(pi),
                                                   log_emit_table=masked)
            out[pre + 'match_i'] = mi
            out[pre + 'match_j'] = mj
            out[pre + 'log_emit'] = np.asarray(masked)
        out[pre + 'log_trans'] = np.asarray(lt)
        out[pre + 'state_types'] = st
        out[pre + 'x'] = x
        out[pre + 'y'] = y
        out[pre + 'sub'] = sub
        out[pre + 'pi'] = pi
        out[pre + 'log_prob'] = np.float64(lp)
        out[pre + 'posteriors'] = np.asarray(post)
        out[pre + 'expected_trans'] = np.asarray(nt)
    path = os.path.join(HERE, 'masked.npz')
    np.savez_compressed(path, **out)
    print('wrote', path, len(out), 'arrays')


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden_masked.py <reference checkout>/python')
    main(sys.argv[1])
