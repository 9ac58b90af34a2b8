"""FP64 oracle: stochastic forward traceback (TEST INFRASTRUCTURE ONLY).

Part of the CPU oracle the test-suite checks the product's sampler
(``phmm_sample_paths``) against; the product never imports it.

Restates ``sample_traceback_2d`` (dp/hmm.py:2043-2101) on the forward table
of ``oracle.dp.forward_table``: the final state drawn with probability
proportional to exp(F[Lx,Ly,s] + logT[s,E]), then, while (i, j) != (0, 0),
the predecessor cell fixed by the current state's type (M: (i-1, j-1), I:
(i, j-1), D: (i-1, j); any other type stops the walk) and its state drawn
proportional to exp(F[pred, s] + logT[s, k]); the path ends with (0, 0, S)
and is returned from the origin on.

The draws use the product's counter-based stream so that paths can be
compared one for one: draw n of sample s of pair p is the top 53 bits of
mix(mix(seed + K (p 2^32 + s)) + K n) / 2^53, mix the SplitMix64 output
function (Steele, Lea and Flood, OOPSLA 2014), K = 0x9e3779b97f4a7c15; a
state is the first index whose running sum of exp(score - max) exceeds u
times the total.  The reference draws with jax.random.choice: other numbers,
the same distribution (checked in the tests against exact path
probabilities).
"""
from __future__ import annotations

import numpy as np

from .dp import forward_table
from .models import M, I, D

MASK = (1 << 64) - 1
K = 0x9e3779b97f4a7c15


def mix64(z):
    z &= MASK
    z = ((z ^ (z >> 30)) * 0xbf58476d1ce4e5b9) & MASK
    z = ((z ^ (z >> 27)) * 0x94d049bb133111eb) & MASK
    return z ^ (z >> 31)


def uniform(stream, n):
    return (mix64(stream + K * n) >> 11) * (1.0 / 9007199254740992.0)


def draw(v, u):
    v = np.asarray(v, float)
    w = np.exp(v - v.max())
    cum = np.cumsum(w)
    hit = np.nonzero(cum > u * cum[-1])[0]
    return int(hit[0]) if hit.size else v.size - 1


def sample_paths(log_trans, state_types, emit, n_samples, seed, pair=0):
    """(log-likelihood, list of n_samples paths [(i, j, state), ...]) of one pair
    with log emission table emit (Lx+1, Ly+1, N); pair is its batch index."""
    lt = np.asarray(log_trans, float)
    st = np.asarray(state_types)
    ll, F = forward_table(lt, st, emit)
    Lx, Ly = F.shape[0] - 1, F.shape[1] - 1
    e_idx = int(np.argmax(st == 4))
    paths = []
    for smp in range(n_samples):
        stream = mix64(seed + K * ((pair << 32) | smp))
        n = 0
        ck = draw(F[Lx, Ly] + lt[:, e_idx], uniform(stream, n))
        n += 1
        ci, cj, path = Lx, Ly, []
        while (ci > 0 or cj > 0) and len(path) < Lx + Ly:
            path.append((ci, cj, ck))
            t = st[ck]
            if t == M and ci > 0 and cj > 0:
                pi_, pj_ = ci - 1, cj - 1
            elif t == I and cj > 0:
                pi_, pj_ = ci, cj - 1
            elif t == D and ci > 0:
                pi_, pj_ = ci - 1, cj
            else:
                break
            ck = draw(F[pi_, pj_] + lt[:, ck], uniform(stream, n))
            n += 1
            ci, cj = pi_, pj_
        path.append((0, 0, 0))
        paths.append(path[::-1])
    return ll, paths
