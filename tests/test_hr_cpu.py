"""Batched Holmes-Rubin statistics (holmes_rubin_batch, the A^3 contraction)
against the per-pair form (holmes_rubin_weighted_stats, the A^4 endpoint
tensor of core/ctmc.py:173-326, itself checked against the reference's
e_step_mixdom2 outputs in test_gpu_api_golden), float64 on the CPU."""
import numpy as np
import torch


def test_batch_matches_per_pair():
    from pairhmm import api, synth
    from pairhmm import models as pm
    rng = np.random.default_rng(5)
    C, P, A = 3, 4, 20
    cls = [synth.rand_Q_pi(rng) for _ in range(C)]
    S = np.stack([c[2] for c in cls])
    pis = np.stack([c[1] for c in cls])
    ts = np.exp(rng.uniform(-3, 1, P))
    mc = rng.gamma(1.0, 2.0, (P, C, A, A))
    W, U = api.holmes_rubin_batch(S, pis, ts, torch.as_tensor(mc))
    for p in range(P):
        for c in range(C):
            Q = pm.build_class_Q(torch.as_tensor(S[c]), torch.as_tensor(pis[c]))
            w, u = api.holmes_rubin_weighted_stats(Q, pis[c], float(ts[p]), mc[p, c])
            np.testing.assert_allclose(W[p, c].numpy(), w.numpy(), rtol=1e-9, atol=1e-12)
            np.testing.assert_allclose(U[p, c].numpy(), u.numpy(), rtol=1e-9, atol=1e-12)
