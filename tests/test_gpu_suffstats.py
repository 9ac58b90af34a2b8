"""Exact MixDom2 sufficient statistics on the GPU: the batched float64
restoration on device tensors against the oracle (1e-12), and the E-step
epilogue end to end (estep_batch_mixdom2(..., exact_suffstats=True)) against
the oracle applied to the oracle's own E-step counts (1e-5 relative to each
output's largest entry: the float32 DP's count bar)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
KEYS = ('top_5x5', 'dom_M_5x5', 'dom_kappa', 'dom_1mkappa', 'ext', 'term', 'dom_w', 'frag_w')


def as_np(v):
    return torch.stack(v, dim=1).cpu().numpy() if isinstance(v, list) else v.cpu().numpy()


@pytest.mark.parametrize('K,F', [(3, 1), (4, 2), (8, 4)])
def test_device_restoration_matches_oracle(cuda_lib, K, F):
    from pairhmm import synth, api
    from oracle import suffstats as osf, models as om
    rng = np.random.default_rng(70 + K * F)
    p = synth.mixdom2_params(rng, K, F, 1)
    B = 4
    ts = np.exp(rng.uniform(-3, 1, B))
    N = 2 + 5 * K * F
    n = np.stack([rng.gamma(1.0, 2.0, (N, N)) *
                  (om.build_nested_trans(p['main_ins'], p['main_del'], ts[b], p['dom_ins'], p['dom_del'],
                                         p['dom_weights'], p['frag_weights'], p['ext_rates']) > 0)
                  for b in range(B)])
    out = api.exact_suffstats_batch(torch.as_tensor(n, device='cuda'), p['main_ins'], p['main_del'], ts,
                                    p['dom_ins'], p['dom_del'], p['dom_weights'], p['frag_weights'],
                                    p['ext_rates'])
    for b in range(B):
        want = osf.exact_suffstats(n[b], p['main_ins'], p['main_del'], ts[b], p['dom_ins'], p['dom_del'],
                                   p['dom_weights'], p['frag_weights'], p['ext_rates'])
        for k in KEYS:
            got = as_np(out[k])[b]
            assert np.abs(got - want[k]).max() <= 1e-12 * max(np.abs(want[k]).max(), 1e-300), k


def test_estep_epilogue_end_to_end(cuda_lib):
    from pairhmm import synth, api
    from oracle import suffstats as osf, estep as oe
    rng = np.random.default_rng(77)
    p = synth.mixdom2_params(rng, 3, 2, 2)
    xs = [rng.integers(0, 20, n) for n in (12, 30, 47)]
    ys = [rng.integers(0, 20, n) for n in (15, 26, 52)]
    ts = np.array([0.2, 0.7, 1.5])
    res = api.estep_batch_mixdom2(p, xs, ys, ts, exact_suffstats=True)
    for b in range(3):
        _, n_or, _ = oe.e_step_mixdom2(dict(p, t=float(ts[b])), xs[b], ys[b])
        want = osf.exact_suffstats(n_or, p['main_ins'], p['main_del'], ts[b], p['dom_ins'], p['dom_del'],
                                   p['dom_weights'], p['frag_weights'], p['ext_rates'])
        for k in KEYS:
            got = as_np(res['suffstats'][k])[b]
            assert np.abs(got - want[k]).max() <= 1e-5 * max(np.abs(want[k]).max(), 1e-300), k
