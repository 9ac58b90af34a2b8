"""FP64 oracle over many pairs on all host cores (TEST INFRASTRUCTURE ONLY).

The C half (oracle/fb2d.c) of the 2D forward-backward, run either as one
single-threaded process per core over a list of pairs (largest first, so the
pool stays balanced) or, for a few large pairs, one pair at a time with every
core on its anti-diagonals.  Processes are started with `spawn`, never forked:
a process forked after the parent touched the GPU can hang.  Used by the
full-size parity tests and bench.py's accuracy leg; the product never imports
it."""
from __future__ import annotations

import os

import numpy as np


def _one(args):
    i, case, forward_only, threads = args
    from oracle import models as om, dp as odp, cdp
    chi, st, groups, EM, EI, ED, x, y = case
    cdp.set_threads(threads)
    emit = odp.log_emission_table(st, groups, x, y, EM, EI, ED)
    if forward_only:
        return i, cdp.forward_backward(om.safe_log(chi), st, emit, True)[0], None, None
    ll, n, cnt = cdp.forward_backward(om.safe_log(chi), st, emit, counts=(groups, EM.shape[0], x, y))
    return i, ll, n, cnt


def estep_pairs(cases, forward_only=False, cores=None):
    """cases: list of (chi, state_types, groups, EM, EI, ED, x, y) with the
    linear model tables of oracle.estep.  Returns one (ll, n_trans, (cM, cI,
    cD)) per case, in order (n_trans and the counts None when forward_only)."""
    import multiprocessing as mp
    from oracle import cdp
    if not cdp.available():
        raise RuntimeError('the C oracle is not built (oracle/build_oracle.py)')
    cores = cores or len(os.sched_getaffinity(0))
    size = lambda c: (len(c[6]) + 1) * (len(c[7]) + 1)
    order = sorted(range(len(cases)), key=lambda i: -size(cases[i]))
    if len(cases) < cores:
        res = [_one((i, cases[i], forward_only, cores)) for i in order]
    else:
        with mp.get_context('spawn').Pool(cores) as pool:
            res = list(pool.imap_unordered(_one, [(i, cases[i], forward_only, 1) for i in order], chunksize=1))
    out = [None] * len(cases)
    for i, ll, n, cnt in res:
        out[i] = (ll, n, cnt)
    return out


def count_errors(got, want):
    """(max |got - want| / max |want|, max relative error over the entries
    above 1e-6 of the largest): the counts bar of the parity tests."""
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    scale = float(np.abs(want).max()) if want.size else 0.0
    if scale <= 0.0:
        return float(np.abs(got).max()) if got.size else 0.0, 0.0
    sig = np.abs(want) > 1e-6 * scale
    return (float(np.abs(got - want).max() / scale),
            float((np.abs(got[sig] - want[sig]) / np.abs(want[sig])).max()) if sig.any() else 0.0)
