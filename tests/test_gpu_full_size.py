"""Parity at the benchmark configurations' real lengths, against the FP64 C
oracle (oracle/fb2d.c through oracle/pool.py, all host cores).

* MixDom2 n_dom=3 n_frag=1 n_classes=1 (17 states): EVERY pair of the
  200-pair LogUniform(30, 600) headline workload (seed 0, longest 599 x 640)
  through the public batched call estep_batch_mixdom2;
* MixDom2 n_dom=4 n_frag=2 n_classes=2 (42 states): one pair of about
  1450 x 1450 (the long end of LogUniform(200, 1500)), E-step outputs and the
  gradient of mixdom2_log_prob; the gradient's reference is the score identity
  evaluated on the ORACLE's counts, differentiated by central differences of
  the oracle's own builders (oracle/models.py), so nothing of the product is
  on the checking side;
* MixDom2 n_dom=8 n_frag=4 n_classes=4 (162 states): one pair of about
  620 x 620 on the wide kernels (20 stripes of 32 rows pipelined through the
  edge rows).

Bars as in the other parity tests: log-likelihood 1e-6 relative; counts 1e-5
relative on the entries above 1e-6 of the largest (and 1e-5 of the largest
in absolute terms); gradients 2e-4 of max(|g|, 1).
"""
import numpy as np
import pytest
import torch

from oracle import models as om, estep as oe, pool

pytestmark = pytest.mark.gpu

LL_RTOL = 1e-6
CNT_RTOL = 1e-5
GRAD_RTOL = 2e-4


def _assert_counts(got, want, what):
    abs_of_max, rel = pool.count_errors(got, want)
    assert rel < CNT_RTOL and abs_of_max <= CNT_RTOL, (what, abs_of_max, rel)


def _cases(w):
    cases = []
    for b in range(len(w.xs)):
        p = dict(w.params)
        p['t'] = float(w.ts[b])
        cases.append(tuple(oe.mixdom2_model(p)[:6]) + (w.xs[b], w.ys[b]))
    return cases


def _check_estep(res, oracle, idx=None):
    host = {k: v.cpu().numpy() for k, v in res.items() if isinstance(v, torch.Tensor)}
    assert (host['status'] == 0).all(), host['status']
    for b, (ll, n, (cM, cI, cD)) in enumerate(oracle):
        assert abs(host['log_p'][b] - ll) <= LL_RTOL * abs(ll), (b, host['log_p'][b], ll)
        _assert_counts(host['n_trans'][b], n, ('n_trans', b))
        _assert_counts(host['cnt_M'][b], cM, ('cnt_M', b))
        _assert_counts(host['cnt_I'][b], cI, ('cnt_I', b))
        _assert_counts(host['cnt_D'][b], cD, ('cnt_D', b))


def test_headline_workload_every_pair(cuda_lib):
    """All 200 pairs of the 17-state headline batch (10.4 M cells)."""
    from pairhmm import api, synth
    w = synth.CONFIGS['mixdom2_k3f1c1_200pairs_len30-600'](seed=0)
    assert max(len(x) for x in w.xs) >= 590 and max(len(y) for y in w.ys) >= 600
    res = api.estep_batch_mixdom2(w.params, w.xs, w.ys, w.ts, with_class_counts=False)
    torch.cuda.synchronize()
    _check_estep(res, pool.estep_pairs(_cases(w)))


def _surrogate(p, t, oracle_one):
    """sum n log chi + sum c log E over one pair with the oracle's counts: its
    gradient in the parameters is the log-likelihood's (score identity)."""
    ll, n, (cM, cI, cD) = oracle_one
    chi, st, groups, EM, EI, ED, _ = oe.mixdom2_model(dict(p, t=t))
    return float((n * om.safe_log(chi)).sum() + (cM * om.safe_log(EM)).sum() + (cI * om.safe_log(EI)).sum()
                 + (cD * om.safe_log(ED)).sum())


def test_42_states_long_pair_estep_and_gradient(cuda_lib):
    from pairhmm import api, synth
    w = synth.make_mixdom2_workload('k4f2c2_long', 4, 2, 2, 1, ('around', 1450, 0.0), seed=11)
    x, y, t = w.xs[0], w.ys[0], float(w.ts[0])
    assert len(x) >= 1400 and len(y) >= 1300, (len(x), len(y))
    oracle = pool.estep_pairs(_cases(w))
    res = api.estep_batch_mixdom2(w.params, w.xs, w.ys, w.ts, with_class_counts=False)
    torch.cuda.synchronize()
    _check_estep(res, oracle)
    # gradient of the log-likelihood through the adjoint
    names = ['main_ins', 'main_del', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates',
             'class_pis', 'class_S_exch', 'classdist']
    p = w.params
    tens = {k: torch.tensor(np.asarray(p[k], float), dtype=torch.float64, requires_grad=True) for k in names}
    tt = torch.tensor([t], dtype=torch.float64, requires_grad=True)
    ll = api.mixdom2_log_prob(tens['main_ins'], tens['main_del'], tt, tens['dom_ins'], tens['dom_del'],
                              tens['dom_weights'], tens['frag_weights'], tens['ext_rates'], tens['class_pis'],
                              tens['class_S_exch'], tens['classdist'], [x], [y])
    ll.sum().backward()
    assert abs(float(ll[0]) - oracle[0][0]) <= LL_RTOL * abs(oracle[0][0])
    rng = np.random.default_rng(0)
    checked = 0
    for k in names + ['t']:
        v = np.asarray(p[k] if k != 't' else t, float)
        flat = v.reshape(-1)
        got_all = (tt.grad.numpy() if k == 't' else tens[k].grad.numpy()).reshape(-1)
        for idx in rng.choice(flat.size, size=min(3, flat.size), replace=False):
            h = 1e-6 * max(abs(flat[idx]), 1e-3)
            a, b = flat.copy(), flat.copy()
            a[idx] += h
            b[idx] -= h
            qa, qb = dict(p), dict(p)
            if k == 't':
                fa, fb = _surrogate(p, float(a[0]), oracle[0]), _surrogate(p, float(b[0]), oracle[0])
            else:
                qa[k] = a.reshape(v.shape) if v.ndim else float(a[0])
                qb[k] = b.reshape(v.shape) if v.ndim else float(b[0])
                fa, fb = _surrogate(qa, t, oracle[0]), _surrogate(qb, t, oracle[0])
            want = (fa - fb) / (2 * h)
            assert abs(got_all[idx] - want) <= GRAD_RTOL * max(abs(want), 1.0), (k, idx, got_all[idx], want)
            checked += 1
    assert checked >= 25


def test_162_states_multi_stripe_pair(cuda_lib):
    from pairhmm import api, synth
    w = synth.make_mixdom2_workload('k8f4c4_long', 8, 4, 4, 1, ('around', 620, 0.0), seed=5)
    assert len(w.xs[0]) >= 600 and len(w.ys[0]) >= 560, (len(w.xs[0]), len(w.ys[0]))
    oracle = pool.estep_pairs(_cases(w))
    res = api.estep_batch_mixdom2(w.params, w.xs, w.ys, w.ts, with_class_counts=False)
    torch.cuda.synchronize()
    _check_estep(res, oracle)
