"""The wide kernels' forward contraction on the tensor cores (phmm_tuning.
tensor = 1: 3xTF32 on mma.sync m16n8k8) for forward-only calls, against the
FP64 C oracle on a multi-stripe pair at 162 states (MixDom2 n_dom=8 n_frag=4
n_classes=4, about 620 x 620): log-likelihood within the 1e-6 relative bar.
An E-step on a plan with the field set runs the float32 contraction and
matches the default bit for bit."""
import numpy as np
import pytest
import torch

from oracle import estep as oe, pool

pytestmark = pytest.mark.gpu


def test_tensor_core_forward_at_162_states(cuda_lib):
    from pairhmm import _lib, api, synth
    from pairhmm import models as pm
    dev = torch.device('cuda')
    w = synth.make_mixdom2_workload('k8f4c4_tc', 8, 4, 4, 2, ('around', 620, 0.0), seed=5)
    K, F, chi, csubs, EM, EI, ED = api._mixdom2_tables(w.params, w.ts, dev)
    cases = []
    for b in range(len(w.xs)):
        p = dict(w.params)
        p['t'] = float(w.ts[b])
        cases.append(tuple(oe.mixdom2_model(p)[:6]) + (w.xs[b], w.ys[b]))
    want = [r[0] for r in pool.estep_pairs(cases, forward_only=True)]
    batch = _lib.make_batch(w.xs, w.ys, chi, EM, EI, ED, device=dev)
    plan = _lib.Plan(pm.mixdom_state_types(K, F), pm.mixdom_state_groups(K, F), K * F)
    ref = _lib.estep(plan, batch)
    plan.set_tuning(tensor=1)
    ll, status = _lib.forward(plan, batch)
    torch.cuda.synchronize()
    assert plan.last_variant == 6 and (status.cpu().numpy() == 0).all()
    for b in range(len(w.xs)):
        assert abs(float(ll[b]) - want[b]) <= 1e-6 * abs(want[b]), (b, float(ll[b]), want[b])
    out = _lib.estep(plan, batch)   # E-steps keep the float32 contraction
    torch.cuda.synchronize()
    assert torch.equal(out['ll'], ref['ll'])
    torch.testing.assert_close(out['n_trans'], ref['n_trans'], rtol=1e-12, atol=1e-12)
