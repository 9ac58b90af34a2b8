"""Captured CUDA graphs of the batched MixDom2 E-step and the autotuner.

* estep_batch_mixdom2 on one batch shape: the first call runs eagerly, the
  second captures the device sequence and later calls replay it.  Every
  replayed call -- with other parameters, other residues of the same lengths
  and times given as a device tensor -- must equal the eager path on the same
  inputs (log-likelihoods bit for bit: the forward recursion is the same
  arithmetic; counts to 1e-12, being sums in another order), and the results
  of a call must survive the next call.
* The autotuner: a tuned plan gives bit-identical log-likelihoods (the
  forward recursion does not depend on the launch configuration), counts
  equal to 1e-6 relative (the float64 atomic sums of the count pass may add
  up in another order), names its configuration, and a later lookup returns
  it.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

KEYS = ('log_p', 'n_trans', 'cnt_M', 'cnt_I', 'cnt_D', 'class_match_counts', 'class_insert_counts',
        'class_delete_counts', 'classdist_counts', 'class_W', 'class_U')


def _eager(api, graphs, params, xs, ys, ts, monkeypatch):
    monkeypatch.setenv('PAIRHMM_GRAPHS', '0')
    try:
        return api.to_host(api.estep_batch_mixdom2(params, xs, ys, ts))
    finally:
        monkeypatch.setenv('PAIRHMM_GRAPHS', '1')


def _same(got, want):
    assert np.array_equal(got['log_p'], want['log_p'])
    assert (got['status'] == 0).all()
    for k in KEYS[1:]:
        np.testing.assert_allclose(got[k], want[k], rtol=1e-12, atol=1e-14 * max(1.0, np.abs(want[k]).max()))


def test_graph_replays_equal_the_eager_path(cuda_lib, monkeypatch):
    from pairhmm import api, graphs, synth
    graphs.clear()
    rng = np.random.default_rng(3)
    w = synth.make_mixdom2_workload('g', 2, 2, 2, 24, ('loguniform', 20, 200), seed=3)
    p2 = synth.mixdom2_params(rng, 2, 2, 2)
    xs2 = [rng.integers(0, 21, len(x)) for x in w.xs]   # other residues, same lengths (wildcards too)
    ys2 = [rng.integers(0, 21, len(y)) for y in w.ys]
    runs = [(w.params, w.xs, w.ys, w.ts), (p2, w.xs, w.ys, w.ts),
            (w.params, xs2, ys2, torch.as_tensor(w.ts[::-1].copy(), device='cuda')), (p2, xs2, ys2, w.ts)]
    kept = None
    for i, (p, xs, ys, ts) in enumerate(runs):
        dev = api.estep_batch_mixdom2(p, xs, ys, ts)
        if i == 1:
            kept = (dev, api.to_host(dev))   # must survive later replays
        got = api.to_host(dev)
        assert (len(graphs._GRAPHS) == 1) == (i >= 1), i
        want = _eager(api, graphs, p, xs, ys, ts.cpu().numpy() if isinstance(ts, torch.Tensor) else ts, monkeypatch)
        _same(got, want)
    _same(api.to_host(kept[0]), kept[1])
    graphs.clear()


def test_autotuned_plan_same_results(cuda_lib, tmp_path, monkeypatch):
    from pairhmm import _lib, api, autotune, synth
    from pairhmm import models as pm
    monkeypatch.setenv('PAIRHMM_TUNE_CACHE', str(tmp_path / 'tuning.json'))
    autotune._MEM.clear()
    w = synth.make_mixdom2_workload('t', 3, 1, 1, 40, ('loguniform', 30, 300), seed=4)
    dev = torch.device('cuda')
    K, F, chi, csubs, EM, EI, ED = api._mixdom2_tables(w.params, w.ts, dev)
    plan = _lib.Plan(pm.mixdom_state_types(K, F), pm.mixdom_state_groups(K, F), K * F)
    b = _lib.make_batch(w.xs, w.ys, chi, EM, EI, ED, device=dev)
    want = _lib.estep(plan, b)
    r = autotune.tune(plan, b, reps=3)
    assert r['evaluated'] >= 5 and r['ms'] <= r['default_ms'] * 1.0001
    assert plan.get_tuning() == r['tuning']
    got = _lib.estep(plan, b)
    torch.cuda.synchronize()
    assert torch.equal(got['ll'], want['ll']) and (got['status'] == 0).all()
    torch.testing.assert_close(got['n_trans'], want['n_trans'], rtol=1e-6, atol=1e-6)
    autotune._MEM.clear()
    plan2 = _lib.Plan(pm.mixdom_state_types(K, F), pm.mixdom_state_groups(K, F), K * F)
    assert autotune.apply_cached(plan2, b) == r['tuning'] and plan2.get_tuning() == r['tuning']
