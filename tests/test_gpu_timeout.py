"""The bounded inter-CTA waits give up cleanly (no GPU fault, no hang).

A plan whose wait bound is cut to one polling iteration (phmm_set_spin_limit)
runs a batch of multi-stripe pairs: a stripe that finds the stripe above (or
below) not yet far enough gives up at once, marks its pair PHMM_ST_TIMEOUT,
releases the stripes waiting on it and returns.  The launch must complete,
every pair must either be exact (status 0, log-likelihood equal to the FP64
oracle's) or marked with the timeout bit and the reference's failure value
NEG_INF = -1e30, at least one pair must have given up, and the next call on
the same plan with the default bound must be exact again.  Nothing here
faults or hangs a GPU: every wait in the kernels has this bound.
"""
import numpy as np
import pytest
import torch

from oracle import estep as oe, pool

pytestmark = pytest.mark.gpu
LL_RTOL = 1e-6
NEG_INF = -1e30


@pytest.mark.parametrize('K,F,C,variant', [(3, 1, 1, 0), (4, 2, 2, 0), (8, 4, 4, 0), (3, 1, 1, 1)])
def test_short_wait_bound_marks_pairs_and_recovers(cuda_lib, K, F, C, variant):
    from pairhmm import _lib, synth
    from pairhmm import models as pm
    rng = np.random.default_rng(17 + K)
    p = synth.mixdom2_params(rng, K, F, C)
    lengths = [(300, 280), (250, 260), (130, 140), (40, 50), (200, 10)] if K * F < 32 else \
        [(100, 90), (70, 80), (20, 30)]
    xs = [rng.integers(0, 20, a) for a, _ in lengths]
    ys = [rng.integers(0, 20, b) for _, b in lengths]
    chi, st, groups, EM, EI, ED, _ = oe.mixdom2_model(p)
    plan = _lib.Plan(st, groups, K * F)
    if variant:
        plan.set_variant(variant)
    b = _lib.make_batch(xs, ys, chi[None], EM[None], EI[None], ED[None], device='cuda')
    want = [r[0] for r in pool.estep_pairs([(chi, st, groups, EM, EI, ED, x, y) for x, y in zip(xs, ys)],
                                           forward_only=True)]
    plan.set_spin_limit(1)
    out = _lib.estep(plan, b)
    torch.cuda.synchronize()
    ll, status = out['ll'].cpu().numpy(), out['status'].cpu().numpy()
    timed_out = (status & 1) != 0
    assert timed_out.any(), status
    for k in range(len(xs)):
        if timed_out[k]:
            assert ll[k] == NEG_INF, (k, ll[k], status[k])
        else:
            assert status[k] == 0 and abs(ll[k] - want[k]) <= LL_RTOL * abs(want[k]), (k, ll[k], want[k])
    plan.set_spin_limit(0)
    out = _lib.estep(plan, b)
    torch.cuda.synchronize()
    assert (out['status'].cpu().numpy() == 0).all()
    ll = out['ll'].cpu().numpy()
    for k in range(len(xs)):
        assert abs(ll[k] - want[k]) <= LL_RTOL * abs(want[k]), (k, ll[k], want[k])
