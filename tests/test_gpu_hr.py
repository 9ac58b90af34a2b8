"""Holmes-Rubin statistics on the GPU (phmm_holmes_rubin: the A^3
contraction through the eigendecomposition of the symmetrised rate matrix)
against the float64 oracle's A^4 endpoint-tensor form (core/ctmc.py:173-326,
oracle.models.holmes_rubin_weighted_stats): 1e-9 relative per entry.  The
reference's own class_W / class_U are checked through e_step_mixdom2 in
test_gpu_api_golden."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _oracle(Q, pis, ts, mc):
    from oracle import models as om
    P, C, A = mc.shape[0], mc.shape[1], mc.shape[2]
    W = np.zeros((P, C, A))
    U = np.zeros((P, C, A, A))
    for p in range(P):
        for c in range(C):
            W[p, c], U[p, c] = om.holmes_rubin_weighted_stats(Q[c], pis[c], float(ts[p]), mc[p, c])
    return W, U


def _check(W, U, Wo, Uo):
    W, U = W.cpu().numpy(), U.cpu().numpy()
    sw, su = np.abs(Wo).max(), np.abs(Uo).max()
    np.testing.assert_allclose(W, Wo, rtol=1e-9, atol=1e-12 * sw)
    np.testing.assert_allclose(U, Uo, rtol=1e-9, atol=1e-12 * su)


@pytest.mark.parametrize('A,C,P', [(20, 3, 7), (4, 2, 5), (20, 1, 200)])
def test_batch_matches_oracle(cuda_lib, A, C, P):
    from pairhmm import api, synth
    rng = np.random.default_rng(500 + A + C + P)
    cls = [synth.rand_Q_pi(rng, A) for _ in range(C)]
    Q = np.stack([c[0] for c in cls])
    pis = np.stack([c[1] for c in cls])
    S = np.stack([c[2] for c in cls])
    ts = np.exp(rng.uniform(np.log(0.01), np.log(5.0), P))
    mc = rng.gamma(1.0, 2.0, (P, C, A, A)) * (rng.random((P, C, A, A)) < 0.5)
    W, U = api.holmes_rubin_batch(S, pis, ts, torch.as_tensor(mc, device='cuda'))
    ridx = rng.choice(P, size=min(P, 12), replace=False)
    Wo, Uo = _oracle(Q, pis, ts[ridx], mc[ridx])
    _check(W[ridx], U[ridx], Wo, Uo)


def test_degenerate_spectrum(cuda_lib):
    """Jukes-Cantor rates (one eigenvalue of multiplicity A-1): the J[k,l]
    rule for equal eigenvalues (t e^{lam t})."""
    from pairhmm import api
    A = 4
    pis = np.full((1, A), 1.0 / A)
    S = np.ones((1, A, A)) * (4.0 / 3.0)
    Q = S * pis[:, None, :]
    np.fill_diagonal(Q[0], 0.0)
    np.fill_diagonal(Q[0], -Q[0].sum(axis=1))
    ts = np.array([1e-3, 0.3, 2.0])
    rng = np.random.default_rng(7)
    mc = rng.gamma(1.0, 1.0, (3, 1, A, A))
    W, U = api.holmes_rubin_batch(S, pis, ts, torch.as_tensor(mc, device='cuda'))
    _check(W, U, *_oracle(Q, pis, ts, mc))
    # dwell times add up to t per unit of count
    np.testing.assert_allclose(W.sum(dim=-1).cpu().numpy()[:, 0], ts * mc.sum(axis=(1, 2, 3)), rtol=1e-12)


def test_single_pair_form(cuda_lib):
    from pairhmm import api, synth
    rng = np.random.default_rng(11)
    Q, pi, _ = synth.rand_Q_pi(rng)
    mc = rng.gamma(1.0, 2.0, (20, 20))
    w, u = api.holmes_rubin_weighted_stats(torch.as_tensor(Q), torch.as_tensor(pi), 0.7, torch.as_tensor(mc))
    from oracle import models as om
    wo, uo = om.holmes_rubin_weighted_stats(Q, pi, 0.7, mc)
    np.testing.assert_allclose(w.numpy(), wo, rtol=1e-9, atol=1e-12 * np.abs(wo).max())
    np.testing.assert_allclose(u.numpy(), uo, rtol=1e-9, atol=1e-12 * np.abs(uo).max())


def test_empty_batch_and_bad_arguments(cuda_lib):
    from pairhmm import _lib
    W, U = _lib.holmes_rubin(np.zeros((1, 4, 4)), np.full((1, 4), 0.25), torch.zeros(0, device='cuda'),
                             torch.zeros(0, 1, 4, 4, dtype=torch.float64, device='cuda'))
    assert W.shape == (0, 1, 4) and U.shape == (0, 1, 4, 4)
    with pytest.raises(_lib.PairHMMError):
        _lib.holmes_rubin(np.zeros((1, 4, 4)), np.array([[0.5, 0.5, 0.0, 0.0]]), torch.ones(1, device='cuda'),
                          torch.zeros(1, 1, 4, 4, dtype=torch.float64, device='cuda'))
