"""Stripe-edge checkpointing of the wide kernels' E-step (phmm_tuning.checkpoint).

The checkpointed E-step keeps only the edge rows between 32-row stripes and
recomputes each stripe's forward and backward recursion from them in the
count pass, in groups of one wave of the recompute kernel (76 stripes on 152
SMs).  It runs the same arithmetic as the full-lattice E-step on the same
inputs, so the log-likelihoods must be bit for bit the same and the counts
equal up to the order of float32 atomic sums (2e-6); against the FP64 oracle the usual bars
hold (LL 1e-6, counts 1e-5).  A batch of 320 stripes runs the count pass in
several groups.  For one 8000 x 8000 pair the scratch it asks for must be a
fraction of the full layout's.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import estep as oe, pool

pytestmark = pytest.mark.gpu
LL_RTOL = 1e-6
CNT_RTOL = 1e-5


def _run(plan, b, checkpoint):
    plan.set_tuning(checkpoint=checkpoint)
    out = {k: v.cpu().numpy() for k, v in __import__('pairhmm')._lib.estep(plan, b).items()}
    torch.cuda.synchronize()
    return out


def _setup(K, F, C, lengths, seed):
    from pairhmm import _lib, synth
    rng = np.random.default_rng(seed)
    p = synth.mixdom2_params(rng, K, F, C)
    chi, st, groups, EM, EI, ED, _ = oe.mixdom2_model(p)
    xs = [rng.integers(0, 20, a) for a, _ in lengths]
    ys = [rng.integers(0, 20, b) for _, b in lengths]
    plan = _lib.Plan(st, groups, K * F)
    b = _lib.make_batch(xs, ys, chi[None], EM[None], EI[None], ED[None], device='cuda')
    return plan, b, (chi, st, groups, EM, EI, ED), xs, ys


def _same(a, b):
    """Log-likelihoods bit for bit (the same forward arithmetic); counts to
    2e-6 (the count pass sums emission posteriors with float32 atomics in
    shared memory, so their order -- and the last bits -- vary from call to
    call in either mode)."""
    assert np.array_equal(a['ll'], b['ll']) and (a['status'] == 0).all() and (b['status'] == 0).all()
    for k in ('n_trans', 'cnt_M', 'cnt_I', 'cnt_D'):
        np.testing.assert_allclose(a[k], b[k], rtol=2e-6, atol=1e-9 * max(1.0, np.abs(b[k]).max()))


@pytest.mark.parametrize('K,F,C', [(8, 4, 4), (4, 4, 1)])
def test_checkpointed_equals_full_and_oracle(cuda_lib, K, F, C):
    lengths = [(100, 90), (70, 80), (33, 31), (32, 32), (0, 5), (6, 0), (1, 1), (64, 10)]
    plan, b, model, xs, ys = _setup(K, F, C, lengths, seed=K + F)
    full = _run(plan, b, 2)
    ck = _run(plan, b, 1)
    _same(ck, full)
    orc = pool.estep_pairs([model + (x, y) for x, y in zip(xs, ys)])
    for k, (ll, n, cnt) in enumerate(orc):
        assert abs(ck['ll'][k] - ll) <= LL_RTOL * abs(ll) + 1e-9, (k, ck['ll'][k], ll)
        for key, want in zip(('n_trans', 'cnt_M', 'cnt_I', 'cnt_D'), (n, *cnt)):
            a, r = pool.count_errors(ck[key][k], want)
            assert a <= CNT_RTOL and r < CNT_RTOL, (k, key, a, r)


def test_checkpointed_several_groups(cuda_lib):
    """40 pairs of 8 stripes each: 320 stripes, several groups."""
    lengths = [(250, 240 + (k % 7)) for k in range(40)]
    plan, b, _, _, _ = _setup(4, 4, 1, lengths, seed=2)
    full = _run(plan, b, 2)
    ck = _run(plan, b, 1)
    _same(ck, full)


def test_checkpointed_scratch_is_small(cuda_lib):
    from pairhmm import _lib
    plan, b, _, _, _ = _setup(8, 4, 4, [(8000, 8000)], seed=1)

    def need(mode):
        plan.set_tuning(checkpoint=mode)
        n = ctypes.c_size_t()
        _lib._check(plan.lib.phmm_workspace_bytes(plan.handle, ctypes.byref(b.struct()), 1, ctypes.byref(n)), 'ws')
        return n.value
    full, ck = need(2), need(1)
    assert ck * 3 < full, (ck, full)
