"""Golden fixtures for the beam-pruned pair-HMM forward-backward, produced by
the reference's own ``dp/hmm_beam.py``: ``msa_to_envelope`` around a guide
alignment, ``beam_forward_2d`` and ``beam_forward_backward_2d`` with and
without an envelope and with finite and infinite beam widths, for TKF91 and a
MixDom model with one substitution model, and ``beam_sample_traceback`` paths
drawn on each case's forward table with a seeded ``numpy.random.RandomState``.

Usage (needs the reference checkout; writes tests/golden/beam.npz):

    python tests/golden/make_golden_beam.py <reference>/python

JAX is replaced by the NumPy stand-in of ``jax_shim.py`` (the beam module
itself is NumPy).  Guide alignments are seeded random M/I/D strings.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import jax_shim  # noqa: E402
from make_golden import rand_Q_pi, rand_mixdom2  # noqa: E402
from make_golden_masked import rand_alignment  # noqa: E402


def main(ref_python):
    jax_shim.install()
    sys.path.insert(0, ref_python)
    from tkfmixdom.jax.dp import hmm_beam as hb
    from tkfmixdom.jax.models import mixdom
    from tkfmixdom.jax.core import params as cp, ctmc
    rng = np.random.default_rng(20261209)
    out = {}
    cases = (('tkf91_env', 'tkf91', 24, 28, np.inf, 3), ('tkf91_beam', 'tkf91', 20, 17, 4.0, None),
             ('tkf91_both', 'tkf91', 30, 33, 6.0, 4), ('mixdom_both', 'mixdom', 15, 18, 5.0, 3),
             ('mixdom_beam', 'mixdom', 12, 10, 2.5, None))
    for name, model, Lx, Ly, beam, bw in cases:
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
        lt = np.log(np.maximum(chi, 1e-300))
        lt[chi <= 0] = -1e30
        x = rng.integers(0, 20, Lx).astype(np.int32)
        y = rng.integers(0, 20, Ly).astype(np.int32)
        env = None
        pre = name + '_'
        if bw is not None:
            _, mx, my = rand_alignment(rng, Lx, Ly)
            env = hb.msa_to_envelope(Lx, Ly, mx, my, bw)
            out[pre + 'msa_x'] = mx
            out[pre + 'msa_y'] = my
            out[pre + 'band_width'] = np.int64(bw)
            out[pre + 'envelope'] = env
        vlp, vpath = hb.beam_viterbi_2d(lt, st, x, y, sub, pi, env)
        out[pre + 'viterbi_log_prob'] = np.float64(vlp)
        out[pre + 'viterbi_path'] = np.asarray(vpath, np.int64)
        lp_f, F_f, n_cells = hb.beam_forward_2d(lt, st, x, y, sub, pi, beam, env)
        lp, post, F = hb.beam_forward_backward_2d(lt, st, x, y, sub, pi, beam, env)
        out[pre + 'log_trans'] = lt
        out[pre + 'state_types'] = st
        out[pre + 'x'] = x
        out[pre + 'y'] = y
        out[pre + 'sub'] = sub
        out[pre + 'pi'] = pi
        out[pre + 'beam'] = np.float64(beam)
        out[pre + 'log_prob'] = np.float64(lp)
        out[pre + 'posteriors'] = np.asarray(post)
        out[pre + 'F'] = np.asarray(F)
        out[pre + 'n_cells'] = np.int64(n_cells)
        assert lp_f == lp
        # four consecutive draws from one seeded RandomState (hmm_beam.py:493-563)
        seed = 1000 + len(out)
        draw = np.random.RandomState(seed)
        paths = [np.asarray(hb.beam_sample_traceback(lt, st, F, lp, x, y, sub, pi, draw, env), np.int64).reshape(-1, 3)
                 for _ in range(4)]
        out[pre + 'sample_seed'] = np.int64(seed)
        out[pre + 'sample_lens'] = np.array([len(q) for q in paths], np.int64)
        out[pre + 'sample_paths'] = np.concatenate(paths)
    # iterative refinement around the diagonal (hmm_beam.py:321-394)
    Q, pi, _ = rand_Q_pi(rng)
    t = 0.5
    lam = 0.03
    chi = np.asarray(cp.tkf91_trans(lam, lam * 1.2, t))
    lt = np.log(np.maximum(chi, 1e-300))
    st = np.array([0, 1, 2, 3, 4])
    sub = np.asarray(ctmc.transition_matrix(Q, t))
    x = rng.integers(0, 20, 26).astype(np.int32)
    y = rng.integers(0, 20, 30).astype(np.int32)
    lp, F, env = hb.iterative_beam_refinement(lt, st, x, y, sub, pi, beam_log_width=8.0, initial_band=3,
                                              n_iterations=3, band_shrink=0.7)
    for k, v in (('log_trans', lt), ('state_types', st), ('x', x), ('y', y), ('sub', sub), ('pi', pi),
                 ('log_prob', np.float64(lp)), ('F', np.asarray(F)), ('envelope', env)):
        out['refine_' + k] = v
    path = os.path.join(HERE, 'beam.npz')
    np.savez_compressed(path, **out)
    print('wrote', path, len(out), 'arrays')


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden_beam.py <reference checkout>/python')
    main(sys.argv[1])
