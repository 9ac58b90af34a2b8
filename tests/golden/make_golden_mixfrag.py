"""Golden outputs of the reference's MixFrag batched E-step and its TKF92
Adam log-likelihood.

Usage (needs the reference checkout; writes tests/golden/mixfrag.npz):

    python tests/golden/make_golden_mixfrag.py <reference>/python

Runs, unmodified under the NumPy stand-in for JAX (``jax_shim.py``):
  * ``estep_batch_mixfrag`` and ``estep_batch_mixfrag_forward_only``
    (``train/mixfrag_svi_bw.py:194-250``) on bin-padded batches of pairs
    with F = 2 and F = 3 fragment types (state spaces of 8 and 11 states);
  * ``tkf92_log_prob_fb`` (``train/tkf92_adam_fb.py:77-104``) on one unpadded
    pair and on padded pairs with real_Lx / real_Ly.
Inputs are stored beside the outputs.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import jax_shim  # noqa: E402
from make_golden import _load_reference, rand_Q_pi, seqs  # noqa: E402


def main(ref_python):
    R = _load_reference(ref_python)
    hmm = R['hmm']
    from tkfmixdom.jax.train import mixfrag_svi_bw as mf, tkf92_adam_fb as adam
    rng = np.random.default_rng(20261205)
    out = {}
    for name, F, lens in (('f2', 2, [(5, 7), (8, 6), (7, 7), (3, 8), (0, 4)]),
                          ('f3', 3, [(6, 5), (9, 9), (4, 7)])):
        Q, pi, _ = rand_Q_pi(rng)
        lam = float(rng.uniform(0.01, 0.05))
        mu = lam * float(rng.uniform(1.05, 1.5))
        exts = rng.uniform(0.3, 0.9, F)
        weights = rng.dirichlet(np.ones(F))
        Lxp = max(hmm._pad_to_bin(a) for a, _ in lens)
        Lyp = max(hmm._pad_to_bin(b) for _, b in lens)
        xs = np.zeros((len(lens), Lxp), np.int32)
        ys = np.zeros((len(lens), Lyp), np.int32)
        for i, (a, b) in enumerate(lens):
            x, y = seqs(rng, a, b)
            xs[i, :a] = x
            ys[i, :b] = y
        ts = np.exp(rng.uniform(np.log(0.1), np.log(1.5), len(lens)))
        Lx = np.array([a for a, _ in lens], np.int32)
        Ly = np.array([b for _, b in lens], np.int32)
        res = mf.estep_batch_mixfrag(xs, ys, ts, Lx, Ly, lam, mu, exts, weights, Q, pi)
        fwd = mf.estep_batch_mixfrag_forward_only(xs, ys, ts, Lx, Ly, lam, mu, exts, weights, Q, pi)
        out.update({f'{name}_{k}': np.asarray(v) for k, v in dict(
            xs=xs, ys=ys, ts=ts, Lx=Lx, Ly=Ly, lam=lam, mu=mu, exts=exts, weights=weights, Q=Q, pi=pi,
            fwd_log_p=np.asarray(fwd)).items()})
        out.update({f'{name}_out_{k}': np.asarray(v, np.float64) for k, v in res.items()})
        print('wrote mixfrag', name, np.asarray(res['log_p']))
    # tkf92_log_prob_fb: one unpadded pair, then padded pairs with real lengths
    Q, pi, _ = rand_Q_pi(rng)
    lam, mu, ext, t = 0.021, 0.03, 0.55, 0.7
    x, y = seqs(rng, 9, 11)
    lp = adam.tkf92_log_prob_fb(lam, mu, ext, t, Q, pi, x, y)
    xp = np.zeros(hmm._pad_to_bin(9), np.int32)
    yp = np.zeros(hmm._pad_to_bin(11), np.int32)
    xp[:9], yp[:11] = x, y
    lp_pad = adam.tkf92_log_prob_fb(lam, mu, ext, t, Q, pi, xp, yp, real_Lx=9, real_Ly=11)
    out.update({'fb_Q': Q, 'fb_pi': pi, 'fb_lam': lam, 'fb_mu': mu, 'fb_ext': ext, 'fb_t': t, 'fb_x': x,
                'fb_y': y, 'fb_xp': xp, 'fb_yp': yp, 'fb_log_p': float(lp), 'fb_log_p_padded': float(lp_pad)})
    print('wrote tkf92_log_prob_fb', float(lp), float(lp_pad))
    np.savez_compressed(os.path.join(HERE, 'mixfrag.npz'), **out)


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden_mixfrag.py <reference checkout>/python')
    main(sys.argv[1])
