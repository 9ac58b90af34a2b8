"""The factored contraction of the two-warp stripes (phmm_batch.nest, the
MixDom chi as exit x top-level-type x dest terms plus same-domain blocks)
against the FP64 oracle and against the dense contraction on the same
batch, through the C ABI.  Bars: LL 1e-6 relative, counts 1e-5 relative
(entries above 1e-6 of the largest)."""
import numpy as np
import pytest
import torch

from oracle import models as om, dp as odp, estep as oe
from test_gpu_kernel_parity import mixdom2_params, related_pair, oracle_estep, assert_counts, LL_RTOL

pytestmark = pytest.mark.gpu

LENGTHS = [(0, 0), (0, 5), (6, 0), (1, 1), (2, 1), (7, 9), (33, 31), (63, 10), (64, 64), (65, 40),
           (40, 97), (130, 120), (129, 3), (300, 280)]


def nested_case(rng, K, F, C, n):
    """n pairs with per-pair times: oracle models and the factored records."""
    from pairhmm import models as pm
    p = mixdom2_params(rng, K, F, C)
    ts = np.exp(rng.uniform(np.log(0.05), np.log(2.0), n))
    cases = []
    for t in ts:
        q = dict(p, t=float(t))
        cases.append(oe.mixdom2_model(q)[:6])
    nest = pm.nested_record(p['main_ins'], p['main_del'], torch.as_tensor(ts), p['dom_ins'], p['dom_del'],
                            p['dom_weights'], p['frag_weights'], p['ext_rates'])
    return cases, nest


def run(cases, xs, ys, nest=None, kf=None, forward_only=False):
    from pairhmm import _lib
    st, groups, EM = cases[0][1], cases[0][2], cases[0][3]
    plan = _lib.Plan(st, groups, EM.shape[0])
    chis = np.stack([c[0] for c in cases])
    EMs, EIs, EDs = (np.stack([c[i] for c in cases]) for i in (3, 4, 5))
    b = _lib.make_batch(xs, ys, chis, EMs, EIs, EDs, nest=nest, nest_kf=kf)
    if forward_only:
        ll, status = _lib.forward(plan, b)
        return {'ll': ll.cpu().numpy(), 'status': status.cpu().numpy()}, plan
    out = _lib.estep(plan, b)
    return {k: v.cpu().numpy() for k, v in out.items()}, plan


@pytest.mark.parametrize('C', [1, 2])
def test_nested_estep_matches_oracle_and_dense(cuda_lib, C):
    rng = np.random.default_rng(101 + C)
    K, F = 3, 1
    cases, nest = nested_case(rng, K, F, C, len(LENGTHS))
    xs, ys = [], []
    for Lx, Ly in LENGTHS:
        x, y = related_pair(rng, Lx, Ly)
        if Lx > 20:
            x[rng.integers(0, Lx, 3)] = 20   # wildcards
        xs.append(x)
        ys.append(y)
    got, plan = run(cases, xs, ys, nest, (K, F))
    assert plan.last_variant == 7
    dense, _ = run(cases, xs, ys)
    assert (got['status'] == 0).all(), got['status']
    for b, (x, y) in enumerate(zip(xs, ys)):
        chi, st, groups, EM, EI, ED = cases[b]
        ll, n, cM, cI, cD = oracle_estep(chi, st, groups, EM, EI, ED, x, y)
        assert abs(got['ll'][b] - ll) <= LL_RTOL * abs(ll) + 1e-9, (b, got['ll'][b], ll)
        assert abs(got['ll'][b] - dense['ll'][b]) <= LL_RTOL * abs(ll) + 1e-9
        assert_counts(got['n_trans'][b], n)
        assert_counts(got['cnt_M'][b], cM)
        assert_counts(got['cnt_I'][b], cI)
        assert_counts(got['cnt_D'][b], cD)


def test_nested_forward_only_and_shared_record(cuda_lib):
    rng = np.random.default_rng(7)
    K, F = 3, 1
    cases, nest = nested_case(rng, K, F, 1, 1)
    pairs = [related_pair(rng, a, b) for a, b in [(0, 3), (50, 61), (200, 190), (1, 0)]]
    xs, ys = [p[0] for p in pairs], [p[1] for p in pairs]
    shared = [cases[0]]   # one chi and one record for every pair
    got, _ = run(shared, xs, ys, nest[:1], (K, F), forward_only=True)
    assert (got['status'] == 0).all()
    chi, st, groups, EM, EI, ED = cases[0]
    for b, (x, y) in enumerate(zip(xs, ys)):
        emit = odp.log_emission_table(st, groups, x, y, EM, EI, ED)
        ll = odp.forward_backward(om.safe_log(chi), st, emit, forward_only=True)[0]
        assert abs(got['ll'][b] - ll) <= LL_RTOL * abs(ll) + 1e-9, (b, got['ll'][b], ll)


def test_nested_record_must_match_the_plan(cuda_lib):
    from pairhmm import _lib
    rng = np.random.default_rng(3)
    cases, nest = nested_case(rng, 3, 1, 1, 1)
    x, y = related_pair(rng, 20, 20)
    with pytest.raises(_lib.PairHMMError, match='nest'):
        run(cases, [x], [y], nest, (2, 1))


@pytest.mark.parametrize('K,F,C', [(3, 1, 1), (4, 2, 2), (8, 4, 4)])
def test_device_record_equals_float64_builder(cuda_lib, K, F, C):
    """phmm_mixdom2_nest (the device prologue) against models.nested_record
    (float64 torch) to float32 rounding."""
    from pairhmm import _lib, models as pm
    rng = np.random.default_rng(5 * K + F)
    p = mixdom2_params(rng, K, F, C)
    ts = np.exp(rng.uniform(np.log(0.05), np.log(2.0), 6))
    pro = _lib.MixDom2Prologue(p)
    got = pro.nest(torch.as_tensor(ts, device='cuda')).cpu().numpy()
    want = pm.nested_record(p['main_ins'], p['main_del'], torch.as_tensor(ts), p['dom_ins'], p['dom_del'],
                            p['dom_weights'], p['frag_weights'], p['ext_rates']).numpy()
    np.testing.assert_allclose(got, want, rtol=2e-7, atol=1e-30)
    assert pro.nest_supported() == ((K, F) == (3, 1) or (F == 4 and 4 <= K <= 8))


WIDE_LENGTHS = [(0, 0), (1, 1), (2, 1), (0, 7), (31, 33), (33, 31), (70, 66), (130, 121)]


def test_wide_nested_estep_matches_oracle_and_dense(cuda_lib):
    """162 states (K=8, F=4) on the wide kernels with the factored record:
    the C oracle and the dense wide kernels on the same batch."""
    from oracle import pool
    rng = np.random.default_rng(77)
    K, F = 8, 4
    cases, nest = nested_case(rng, K, F, 2, len(WIDE_LENGTHS))
    xs, ys = [], []
    for Lx, Ly in WIDE_LENGTHS:
        x, y = related_pair(rng, Lx, Ly)
        xs.append(x)
        ys.append(y)
    got, plan = run(cases, xs, ys, nest, (K, F))
    assert plan.last_variant == 6
    dense, _ = run(cases, xs, ys)
    assert (got['status'] == 0).all(), got['status']
    oracle = pool.estep_pairs([tuple(c) + (x, y) for c, x, y in zip(cases, xs, ys)])
    for b, (ll, n, (cM, cI, cD)) in enumerate(oracle):
        assert abs(got['ll'][b] - ll) <= LL_RTOL * abs(ll) + 1e-9, (b, got['ll'][b], ll)
        assert abs(got['ll'][b] - dense['ll'][b]) <= LL_RTOL * abs(ll) + 1e-9
        assert_counts(got['n_trans'][b], n)
        assert_counts(got['cnt_M'][b], cM)
        assert_counts(got['cnt_I'][b], cI)
        assert_counts(got['cnt_D'][b], cD)
    fwd, _ = run(cases, xs, ys, nest, (K, F), forward_only=True)
    for b, (ll, _, _) in enumerate(oracle):
        assert abs(fwd['ll'][b] - ll) <= LL_RTOL * abs(ll) + 1e-9, (b, fwd['ll'][b], ll)
