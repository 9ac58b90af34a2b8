"""Float64 BDI epilogue of the batched TKF92 E-step (pairhmm.bdi, torch
autograd) against the oracle restatement (complex-step derivatives), on the
CPU: general branch, the L'Hopital branch at lambda = mu, and the chi
decomposition."""
import numpy as np
import pytest
import torch

from oracle import bdi as ob
from pairhmm import bdi


def _counts(rng, B):
    n = rng.uniform(0.0, 3.0, (B, 5, 5))
    n[:, :, 0] = 0.0        # nothing enters the start state
    n[:, 4, :] = 0.0        # nothing leaves the end state
    return n


@pytest.mark.parametrize('lam,mu', [(0.02, 0.03), (0.04, 0.041), (0.05, 0.05)])
def test_bdi_stats_match_oracle(lam, mu):
    rng = np.random.default_rng(3)
    n = _counts(rng, 6)
    t = rng.uniform(0.1, 2.0, 6)
    EB, ED, ES = bdi.bdi_stats(torch.tensor(n), lam, mu, torch.tensor(t))
    for b in range(6):
        want = ob.bdi_stats(n[b], lam, mu, t[b])
        got = (float(EB[b]), float(ED[b]), float(ES[b]))
        tol = 1e-6 if lam != mu else 1e-5   # the limit branch's oracle uses a central difference
        for g, w in zip(got, want):
            assert abs(g - w) <= tol * max(abs(w), 1.0), (b, got, want)


def test_tkf92_epilogue_matches_oracle():
    rng = np.random.default_rng(5)
    n = _counts(rng, 4)
    t = rng.uniform(0.1, 2.0, 4)
    lam, mu, ext = 0.03, 0.04, 0.6
    out = bdi.tkf92_bdi_epilogue(torch.tensor(n), lam, mu, torch.tensor(t), ext)
    for b in range(4):
        want = ob.tkf92_epilogue(n[b], lam, mu, t[b], ext)
        for k, w in want.items():
            assert abs(float(out[k][b]) - w) <= 1e-9 * max(abs(w), 1.0), (k, b, float(out[k][b]), w)
    np.testing.assert_allclose(out['T'].numpy(), t)
