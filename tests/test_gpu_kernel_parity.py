"""CUDA E-step kernel vs the FP64 oracle, through the C ABI.

Bars: per-pair log-likelihood within 1e-6 relative,
expected counts within 1e-5 relative (entries above 1e-6 of the largest).
The kernel runs in float32 probability space; the oracle in float64 log space.
"""
import numpy as np
import pytest

from oracle import models as om, dp as odp, estep as oe

LL_RTOL = 1e-6
CNT_RTOL = 1e-5

pytestmark = pytest.mark.gpu


def rand_Q_pi(rng, A=20):
    pi = rng.dirichlet(np.ones(A))
    Sx = rng.lognormal(0.0, 1.0, size=(A, A))
    Sx = np.triu(Sx, 1)
    Sx = Sx + Sx.T
    Q = Sx * pi[None, :]
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(axis=1))
    rate = -np.sum(pi * np.diag(Q))
    return Q / rate, pi, Sx / rate


def mixdom2_params(rng, K, F, C):
    cls = [rand_Q_pi(rng) for _ in range(C)]
    p = {'main_ins': rng.uniform(0.01, 0.05), 't': float(np.exp(rng.uniform(np.log(0.05), np.log(2.0)))),
         'dom_ins': rng.uniform(0.01, 0.05, K), 'dom_weights': rng.dirichlet(np.ones(K)),
         'frag_weights': np.stack([rng.dirichlet(np.ones(F)) for _ in range(K)]),
         'class_pis': np.stack([c[1] for c in cls]), 'class_S_exch': np.stack([c[2] for c in cls]),
         'classdist': np.stack([[rng.dirichlet(np.ones(C)) for _ in range(F)] for _ in range(K)]),
         'ext_rates': rng.uniform(0.3, 0.9, (K, F))}
    p['main_del'] = p['main_ins'] * rng.uniform(1.05, 1.5)
    p['dom_del'] = p['dom_ins'] * rng.uniform(1.05, 1.5, K)
    return p


def oracle_case(model, rng, K=3, F=1, C=1):
    if model == 'tkf91':
        Q, pi, _ = rand_Q_pi(rng)
        lam = rng.uniform(0.01, 0.05)
        p = {'ins_rate': lam, 'del_rate': lam * rng.uniform(1.05, 1.5), 't': rng.uniform(0.1, 1.5),
             'Q': Q, 'pi': pi}
        chi, st, groups, EM, EI, ED, _ = oe.tkf_model('tkf91', p)
    else:
        p = mixdom2_params(rng, K, F, C)
        chi, st, groups, EM, EI, ED, _ = oe.mixdom2_model(p)
    return chi, st, groups, EM, EI, ED


def related_pair(rng, Lx, Ly):
    """A descendant that shares most residues with the ancestor (realistic LL scale)."""
    x = rng.integers(0, 20, Lx)
    y = np.array([x[int(k * Lx / max(Ly, 1))] if Lx and rng.random() < 0.7 else rng.integers(0, 20)
                  for k in range(Ly)], dtype=np.int64)
    return x, y


def run_kernel(chi, st, groups, EM, EI, ED, xs, ys, per_pair=None, variant=0):
    """per_pair: optional list of (chi, EM, EI, ED) per pair; variant 1 =
    generic kernels, 2 = register-resident warp kernels, 3 = block kernels,
    4 = split warp E-step, 5 = split block E-step, 6 = wide kernels, 7 = split
    E-step on two-warp stripes, 0 = automatic."""
    from pairhmm import _lib
    G = EM.shape[0]
    plan = _lib.Plan(st, groups, G)
    if variant:
        try:
            plan.set_variant(variant)
        except _lib.PairHMMError:
            pytest.skip('no kernel of this family for the state space')
    if per_pair is not None:
        chis, EMs, EIs, EDs = (np.stack(v) for v in zip(*per_pair))
    else:
        chis, EMs, EIs, EDs = chi[None], EM[None], EI[None], ED[None]
    b = _lib.make_batch(xs, ys, chis, EMs, EIs, EDs)
    out = _lib.estep(plan, b)
    if variant:
        assert plan.last_variant == variant
    return {k: v.cpu().numpy() for k, v in out.items()}, plan


def oracle_estep(chi, st, groups, EM, EI, ED, x, y):
    emit = odp.log_emission_table(st, groups, x, y, EM, EI, ED)
    ll, post, n, F, B = odp.forward_backward(om.safe_log(chi), st, emit)
    cM, cI, cD = oe.char_count_tables(post, st, groups, x, y, EM.shape[0])
    return ll, n, cM, cI, cD


def assert_counts(got, want, rtol=CNT_RTOL):
    want = np.asarray(want)
    got = np.asarray(got)
    scale = np.abs(want).max() if want.size else 0.0
    sig = np.abs(want) > 1e-6 * max(scale, 1e-300)
    if sig.any():
        rel = np.abs(got[sig] - want[sig]) / np.abs(want[sig])
        assert rel.max() < rtol, f'max rel count error {rel.max():.3e}'
    assert np.abs(got - want).max() <= max(rtol * scale, 1e-12)


LENGTHS = [(0, 0), (0, 5), (6, 0), (1, 1), (7, 9), (31, 33), (32, 32), (33, 31),
           (63, 10), (64, 64), (65, 40), (40, 97), (130, 120), (129, 3)]


@pytest.mark.parametrize('variant', [1, 2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize('model,K,F,C', [('tkf91', 1, 1, 1), ('mixdom2', 3, 1, 1),
                                         ('mixdom2', 2, 2, 2), ('mixdom2', 4, 2, 2),
                                         ('mixdom2', 1, 1, 2), ('mixdom2', 2, 1, 1)])
def test_estep_matches_oracle(cuda_lib, model, K, F, C, variant):
    rng = np.random.default_rng(7 + K * 10 + F + C)
    chi, st, groups, EM, EI, ED = oracle_case(model, rng, K, F, C)
    xs, ys = [], []
    for Lx, Ly in LENGTHS:
        x, y = related_pair(rng, Lx, Ly)
        xs.append(x)
        ys.append(y)
    out, _ = run_kernel(chi, st, groups, EM, EI, ED, xs, ys, variant=variant)
    assert (out['status'] == 0).all(), out['status']
    for b, (x, y) in enumerate(zip(xs, ys)):
        ll, n, cM, cI, cD = oracle_estep(chi, st, groups, EM, EI, ED, x, y)
        assert abs(out['ll'][b] - ll) <= LL_RTOL * abs(ll) + 1e-9, (b, out['ll'][b], ll)
        assert_counts(out['n_trans'][b], n)
        assert_counts(out['cnt_M'][b], cM)
        assert_counts(out['cnt_I'][b], cI)
        assert_counts(out['cnt_D'][b], cD)


@pytest.mark.parametrize('variant', [7])
def test_two_warp_forward_only_matches_oracle(cuda_lib, variant):
    """phmm_forward on the two-warp stripe kernels (variant 7)."""
    from pairhmm import _lib
    rng = np.random.default_rng(11)
    chi, st, groups, EM, EI, ED = oracle_case('mixdom2', rng, 3, 1, 1)
    xs, ys = zip(*[related_pair(rng, a, b) for a, b in LENGTHS + [(200, 150)]])
    plan = _lib.Plan(st, groups, EM.shape[0])
    plan.set_variant(variant)
    b = _lib.make_batch(xs, ys, chi[None], EM[None], EI[None], ED[None])
    ll_f, st_f = _lib.forward(plan, b)
    assert plan.last_variant == variant
    assert (st_f.cpu().numpy() == 0).all()
    for k, (x, y) in enumerate(zip(xs, ys)):
        ll = oracle_estep(chi, st, groups, EM, EI, ED, x, y)[0]
        assert abs(ll_f[k].item() - ll) <= LL_RTOL * abs(ll) + 1e-9, (k, ll_f[k].item(), ll)


def test_forward_only_matches_estep_ll(cuda_lib):
    from pairhmm import _lib
    rng = np.random.default_rng(3)
    chi, st, groups, EM, EI, ED = oracle_case('mixdom2', rng, 3, 1, 1)
    xs, ys = zip(*[related_pair(rng, a, b) for a, b in LENGTHS])
    plan = _lib.Plan(st, groups, EM.shape[0])
    b = _lib.make_batch(xs, ys, chi[None], EM[None], EI[None], ED[None])
    ll_f, st_f = _lib.forward(plan, b)
    out = _lib.estep(plan, b)
    assert (st_f.cpu().numpy() == 0).all()
    np.testing.assert_array_equal(ll_f.cpu().numpy(), out['ll'].cpu().numpy())


@pytest.mark.parametrize('variant', [1, 2, 3, 4, 5, 6, 7])
def test_per_pair_chi_and_wildcards(cuda_lib, variant):
    rng = np.random.default_rng(11)
    base = mixdom2_params(rng, 2, 1, 1)
    xs, ys, per_pair, lls = [], [], [], []
    for b, (Lx, Ly) in enumerate([(20, 25), (50, 45), (3, 70)]):
        p = dict(base)
        p['t'] = [0.1, 0.7, 1.9][b]
        chi, st, groups, EM, EI, ED, _ = oe.mixdom2_model(p)
        x, y = related_pair(rng, Lx, Ly)
        x[::7] = 20
        y[::5] = 20
        xs.append(x)
        ys.append(y)
        per_pair.append((chi, EM, EI, ED))
        lls.append(oracle_estep(chi, st, groups, EM, EI, ED, x, y))
    # t changes both chi and the class P_c(t) tables: one set per pair
    out, _ = run_kernel(None, st, groups, EM, EI, ED, xs, ys, per_pair=per_pair, variant=variant)
    for b in range(3):
        ll, n, cM, cI, cD = lls[b]
        assert abs(out['ll'][b] - ll) <= LL_RTOL * abs(ll)
        assert_counts(out['n_trans'][b], n)
        assert_counts(out['cnt_M'][b], cM)


@pytest.mark.parametrize('variant', [1, 2, 3, 4, 5, 6, 7])
def test_long_pair_pipelined_stripes(cuda_lib, variant):
    """A pair spanning many stripes (pipelined through the edge rows), against the oracle."""
    rng = np.random.default_rng(5)
    chi, st, groups, EM, EI, ED = oracle_case('mixdom2', rng, 3, 1, 1)
    x, y = related_pair(rng, 300, 280)
    out, _ = run_kernel(chi, st, groups, EM, EI, ED, [x], [y], variant=variant)
    ll, n, cM, cI, cD = oracle_estep(chi, st, groups, EM, EI, ED, x, y)
    assert abs(out['ll'][0] - ll) <= LL_RTOL * abs(ll)
    assert_counts(out['n_trans'][0], n)
    assert_counts(out['cnt_D'][0], cD)


# Large state spaces (more than 64 padded slots) run on the wide kernels:
# n_dom=4 n_frag=4 (82 states), n_dom=13 n_frag=1 (67 states: the start state
# shares the last M quad), n_dom=8 n_frag=4 n_classes=4 (162 states).
WIDE_LENGTHS = [(0, 0), (0, 5), (6, 0), (1, 1), (9, 7), (31, 33), (32, 32), (33, 31), (64, 10), (20, 65)]


@pytest.mark.parametrize('K,F,C', [(4, 4, 1), (13, 1, 1), (8, 4, 4)])
def test_wide_state_spaces_match_oracle(cuda_lib, K, F, C):
    rng = np.random.default_rng(100 + K + F + C)
    chi, st, groups, EM, EI, ED = oracle_case('mixdom2', rng, K, F, C)
    lengths = WIDE_LENGTHS if K * F < 32 else WIDE_LENGTHS[:8]
    xs, ys = zip(*[related_pair(rng, a, b) for a, b in lengths])
    out, plan = run_kernel(chi, st, groups, EM, EI, ED, list(xs), list(ys))
    assert plan.last_variant == 6
    assert (out['status'] == 0).all(), out['status']
    for b, (x, y) in enumerate(zip(xs, ys)):
        ll, n, cM, cI, cD = oracle_estep(chi, st, groups, EM, EI, ED, x, y)
        assert abs(out['ll'][b] - ll) <= LL_RTOL * abs(ll) + 1e-9, (b, out['ll'][b], ll)
        assert_counts(out['n_trans'][b], n)
        assert_counts(out['cnt_M'][b], cM)
        assert_counts(out['cnt_I'][b], cI)
        assert_counts(out['cnt_D'][b], cD)


def test_wide_forward_only_and_long_pair(cuda_lib):
    """phmm_forward on the wide kernels, and a pair spanning many 32-row stripes."""
    from pairhmm import _lib
    rng = np.random.default_rng(21)
    chi, st, groups, EM, EI, ED = oracle_case('mixdom2', rng, 4, 4, 1)
    x, y = related_pair(rng, 100, 90)
    plan = _lib.Plan(st, groups, EM.shape[0])
    b = _lib.make_batch([x], [y], chi[None], EM[None], EI[None], ED[None])
    ll_f, st_f = _lib.forward(plan, b)
    out = _lib.estep(plan, b)
    ll, n, cM, cI, cD = oracle_estep(chi, st, groups, EM, EI, ED, x, y)
    assert int(st_f.cpu()[0]) == 0
    assert abs(float(ll_f.cpu()[0]) - ll) <= LL_RTOL * abs(ll)
    assert abs(float(out['ll'].cpu()[0]) - ll) <= LL_RTOL * abs(ll)
    assert_counts(out['n_trans'][0].cpu().numpy(), n)
    assert_counts(out['cnt_M'][0].cpu().numpy(), cM)
