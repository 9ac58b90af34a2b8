"""MixFrag batched E-step epilogue and TKF92 Adam log-likelihood on the CPU,
against the reference's own outputs (tests/golden/mixfrag.npz, made by
tests/golden/make_golden_mixfrag.py from train/mixfrag_svi_bw.py and
train/tkf92_adam_fb.py): the FP64 oracle's forward-backward counts go through
the float64 resolution and BDI epilogue of pairhmm.bdi, which must give the
reference's B, D, S, L, M, F_f, E_f; the batched torch builder of the MixFrag
matrix equals the oracle's."""
import numpy as np
import pytest
import torch

from conftest import GOLDEN
from oracle import models as om, dp as odp, cdp

G = np.load(GOLDEN + '/mixfrag.npz')


def _oracle_case(name, b):
    F = G[f'{name}_exts'].size
    chi = np.maximum(om.mixfrag_trans(float(G[f'{name}_lam']), float(G[f'{name}_mu']), float(G[f'{name}_ts'][b]),
                                      G[f'{name}_exts'], G[f'{name}_weights']), 1e-30)
    st = np.array([0] + [1] * F + [2] * F + [3] * F + [4])
    sub = om.transition_matrix(G[f'{name}_Q'], float(G[f'{name}_ts'][b]))
    EM, EI, ED = odp.group_tables_tkf(sub, G[f'{name}_pi'])
    Lx, Ly = int(G[f'{name}_Lx'][b]), int(G[f'{name}_Ly'][b])
    x, y = G[f'{name}_xs'][b, :Lx].astype(int), G[f'{name}_ys'][b, :Ly].astype(int)
    emit = odp.log_emission_table(st, np.zeros(st.size, int), x, y, EM, EI, ED)
    return chi, st, emit


@pytest.mark.parametrize('name', ['f2', 'f3'])
def test_mixfrag_epilogue_matches_reference(name):
    from pairhmm import bdi
    from pairhmm import models as pm
    P = G[f'{name}_ts'].size
    ns, lls = [], []
    for b in range(P):
        chi, st, emit = _oracle_case(name, b)
        ll, post, n, _, _ = odp.forward_backward(om.safe_log(chi), st, emit)
        ns.append(n)
        lls.append(ll)
    np.testing.assert_allclose(lls, G[f'{name}_out_log_p'], rtol=1e-12)
    np.testing.assert_allclose(lls, G[f'{name}_fwd_log_p'], rtol=1e-12)
    res = bdi.mixfrag_bdi_epilogue(torch.as_tensor(np.stack(ns)), float(G[f'{name}_lam']), float(G[f'{name}_mu']),
                                   G[f'{name}_ts'], G[f'{name}_exts'], G[f'{name}_weights'])
    # B, D, S pass through the reference's jax.grad of its BDI likelihood, a
    # Richardson-extrapolated difference in the stand-in (~1e-9), which E[S]
    # divides by (lambda - mu): ~2e-7 in the fixture
    for k in ('B', 'D', 'S', 'L', 'M', 'T', 'F_f', 'E_f'):
        rtol = 1e-6 if k in 'BDS' else 1e-9
        np.testing.assert_allclose(res[k].numpy(), G[f'{name}_out_{k}'], rtol=rtol, atol=1e-12, err_msg=k)
    chi_b = pm.mixfrag_trans_batch(float(G[f'{name}_lam']), float(G[f'{name}_mu']), torch.as_tensor(G[f'{name}_ts']),
                                   G[f'{name}_exts'], G[f'{name}_weights']).numpy()
    for b in range(P):
        want = om.mixfrag_trans(float(G[f'{name}_lam']), float(G[f'{name}_mu']), float(G[f'{name}_ts'][b]),
                                G[f'{name}_exts'], G[f'{name}_weights'])
        np.testing.assert_allclose(chi_b[b], want, rtol=1e-13, atol=1e-300)


def test_tkf92_log_prob_fb_reference_value():
    """The reference's TKF92 Adam likelihood equals the oracle's TKF92
    forward with the 1e-30 floor, padded or not."""
    chi = np.maximum(om.tkf92_trans(G['fb_lam'], G['fb_mu'], G['fb_t'], G['fb_ext']), 1e-30)
    sub = om.transition_matrix(G['fb_Q'], float(G['fb_t']))
    EM, EI, ED = odp.group_tables_tkf(sub, G['fb_pi'])
    st = om.tkf_state_types()
    emit = odp.log_emission_table(st, np.zeros(5, int), G['fb_x'].astype(int), G['fb_y'].astype(int), EM, EI, ED)
    ll = odp.forward_table(om.safe_log(chi), st, emit)[0]
    assert abs(ll - float(G['fb_log_p'])) < 1e-12 * abs(ll)
    assert float(G['fb_log_p_padded']) == float(G['fb_log_p'])
