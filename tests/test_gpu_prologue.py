"""Device prologues of the MixDom2 and TKF92 E-steps (phmm_mixdom2_tables,
phmm_tkf92_tables) and the class-count epilogue against the
float64 torch builders, which the oracle tests pin to the reference.

Bars: chi and the emission tables are float32 roundings of float64 values,
so they agree to a few float32 ulps (rtol 1e-6), up to float64 cancellation
in entries far below 1 (atol 1e-14: at t = 1e-6 both float64 builders differ
by 5e-16 on entries of 2e-10); P_c(t) is float64 on both sides (Pade-13
scaling and squaring here, torch.linalg.matrix_exp there) and agrees to rtol
1e-11 on entries above 1e-14 and to 1e-12 absolute (t = 400 takes 8
squarings).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
F32_RTOL = 1e-6
EXPM_RTOL = 1e-11


def torch_tables(p, ts):
    from pairhmm import models as pm
    t = torch.as_tensor(np.asarray(ts, np.float64))
    chi = pm.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'], p['dom_weights'],
                                p['frag_weights'], p['ext_rates'])
    cs = pm.class_subs(pm._t(p['class_S_exch']), pm._t(p['class_pis']), t)
    EM, EI, ED = pm.tables_per_class(cs, pm._t(p['class_pis']), pm._t(p['classdist']))
    return chi, cs, EM, EI, ED


def check(p, ts):
    from pairhmm import _lib
    chi, EM, EI, ED, cs = _lib.mixdom2_tables(p, ts, device='cuda')
    rchi, rcs, rEM, rEI, rED = torch_tables(p, ts)
    torch.testing.assert_close(chi.cpu(), rchi.float(), rtol=F32_RTOL, atol=1e-14)
    big = rcs.abs() > 1e-14
    rel = ((cs.cpu() - rcs).abs() / rcs.abs().clamp_min(1e-300))[big]
    assert rel.max().item() < EXPM_RTOL, rel.max().item()
    assert (cs.cpu() - rcs).abs().max().item() < 1e-12
    torch.testing.assert_close(EM.cpu(), rEM.float(), rtol=F32_RTOL, atol=1e-30)
    torch.testing.assert_close(EI.cpu(), rEI.float().expand_as(EI.cpu()), rtol=F32_RTOL, atol=1e-30)
    torch.testing.assert_close(ED.cpu(), rED.float().expand_as(ED.cpu()), rtol=F32_RTOL, atol=1e-30)


@pytest.mark.parametrize('K,F,C', [(3, 1, 1), (4, 2, 2), (8, 4, 4), (1, 1, 3), (11, 3, 2)])
def test_prologue_matches_float64_builders(cuda_lib, K, F, C):
    from pairhmm import synth
    rng = np.random.default_rng(100 + 7 * K + F + C)
    p = synth.mixdom2_params(rng, K, F, C)
    # times from no scaling (||tQ|| below theta_13) to many squarings
    ts = np.concatenate([[1e-6, 1e-3, 0.05, 1.0, 4.0, 40.0, 400.0], np.exp(rng.uniform(-3, 1, 25))])
    check(p, ts)


def test_prologue_full_fragment_extension_matrix(cuda_lib):
    """ext_rates given as a [K][F][F] matrix with off-diagonal extensions."""
    from pairhmm import synth
    rng = np.random.default_rng(5)
    K, F = 3, 3
    p = synth.mixdom2_params(rng, K, F, 2)
    ext = rng.uniform(0.02, 0.25, (K, F, F))
    p['ext_rates'] = ext
    check(p, np.exp(rng.uniform(-3, 1, 16)))


def test_prologue_equal_rate_branches(cuda_lib):
    """lambda ~ mu at the main and domain levels takes the limit forms."""
    from pairhmm import synth
    rng = np.random.default_rng(9)
    p = synth.mixdom2_params(rng, 4, 2, 1)
    p['main_del'] = p['main_ins'] * (1 + 1e-6)
    p['dom_del'] = p['dom_ins'].copy()
    p['dom_del'][0] = p['dom_ins'][0] * (1 + 3e-5)   # inside the 1e-4 band
    p['dom_del'][1] = p['dom_ins'][1] * (1 + 3e-4)   # just outside it
    check(p, np.exp(rng.uniform(-4, 1, 12)))


def test_batched_estep_through_the_prologue_matches_oracle(cuda_lib):
    """estep_batch_mixdom2 (device prologue + E-step) against the float64 oracle."""
    from pairhmm import synth, api
    from oracle import estep as oe
    rng = np.random.default_rng(21)
    K, F, C = 3, 2, 2
    p = synth.mixdom2_params(rng, K, F, C)
    xs = [rng.integers(0, 20, n) for n in (1, 17, 40, 66)]
    ys = [rng.integers(0, 20, n) for n in (3, 25, 38, 70)]
    ts = np.array([0.1, 0.5, 1.2, 2.0])
    out = api.estep_batch_mixdom2(p, xs, ys, ts)
    for b in range(len(xs)):
        q = dict(p, t=float(ts[b]))
        ll, nt, _ = oe.e_step_mixdom2(q, xs[b], ys[b])
        assert abs(out['log_p'][b].item() - ll) <= 1e-6 * abs(ll)
        want = np.asarray(nt)
        got = out['n_trans'][b].cpu().numpy()
        scale = np.abs(want).max()
        assert np.abs(got - want).max() <= 1e-5 * scale


@pytest.mark.parametrize('K,F,C', [(3, 1, 1), (4, 2, 2), (8, 4, 4), (2, 3, 8)])
def test_class_count_epilogue_matches_torch(cuda_lib, K, F, C):
    """phmm_mixdom2_class_counts against the float64 torch class split."""
    from pairhmm import synth, api, _lib
    rng = np.random.default_rng(40 + K * F * C)
    p = synth.mixdom2_params(rng, K, F, C)
    P, G = 6, K * F
    ts = np.exp(rng.uniform(-3, 1, P))
    pro = _lib.MixDom2Prologue(p)
    _, _, _, _, cs = pro(ts, device='cuda')
    cM = torch.as_tensor(rng.gamma(1.0, 3.0, (P, G, 21, 21)), device='cuda')
    cI = torch.as_tensor(rng.gamma(1.0, 3.0, (P, G, 21)), device='cuda')
    cD = torch.as_tensor(rng.gamma(1.0, 3.0, (P, G, 21)), device='cuda')
    got = pro.class_counts(cs, cM, cI, cD)
    want = api.class_split(p, cM, cI, cD, csubs=cs)
    for k, v in want.items():
        torch.testing.assert_close(got[k], v, rtol=1e-12, atol=1e-12, msg=k)


@pytest.mark.parametrize('ext,equal_rates', [(0.0, False), (0.4, False), (0.3, True)])
def test_tkf92_prologue_matches_float64_builders(cuda_lib, ext, equal_rates):
    """phmm_tkf92_tables against the float64 torch builders of the batched
    TKF92 path (chi floored at 1e-30, expm(t Q), pair-HMM emission tables)."""
    from pairhmm import synth, _lib
    from pairhmm import models as pm
    rng = np.random.default_rng(31 + int(10 * ext) + int(equal_rates))
    p = synth.tkf_params(rng, ext=ext)
    if equal_rates:
        p['del_rate'] = p['ins_rate'] * (1 + 1e-6)
    ts = np.concatenate([[1e-6, 0.01, 1.0, 30.0], np.exp(rng.uniform(-3, 1, 12))])
    chi, EM, EI, ED, sub = _lib.tkf92_tables(p['ins_rate'], p['del_rate'], ext, p['Q'], p['pi'], ts,
                                             device='cuda')
    t = torch.as_tensor(ts)
    rchi = pm.tkf92_trans(p['ins_rate'], p['del_rate'], t, ext).clamp_min(1e-30)
    rsub = pm.transition_matrix(pm._t(p['Q']), t)
    rEM, rEI, rED = pm.tables_tkf(rsub, pm._t(p['pi']))
    torch.testing.assert_close(chi.cpu(), rchi.float(), rtol=F32_RTOL, atol=1e-14)
    big = rsub.abs() > 1e-14
    rel = ((sub.cpu() - rsub).abs() / rsub.abs().clamp_min(1e-300))[big]
    assert rel.max().item() < EXPM_RTOL, rel.max().item()
    torch.testing.assert_close(EM.cpu(), rEM.float(), rtol=F32_RTOL, atol=1e-14)
    torch.testing.assert_close(EI.cpu(), rEI.float().expand_as(EI.cpu()), rtol=F32_RTOL, atol=1e-14)
    torch.testing.assert_close(ED.cpu(), rED.float().expand_as(ED.cpu()), rtol=F32_RTOL, atol=1e-14)


@pytest.mark.parametrize('K,F,full_ext,equal_rates', [(3, 1, False, False), (4, 2, False, False),
                                                      (2, 3, True, False), (3, 2, False, True)])
def test_chi_vjp_matches_autograd(cuda_lib, K, F, full_ext, equal_rates):
    """The device chi VJP (forward-mode duals) against torch autograd through
    the float64 builder, for every chi parameter and the per-pair times."""
    from pairhmm import synth, api, _lib
    from pairhmm import models as pm
    rng = np.random.default_rng(60 + K * F + int(full_ext) + 2 * int(equal_rates))
    p = synth.mixdom2_params(rng, K, F, 1)
    if full_ext:
        p['ext_rates'] = rng.uniform(0.02, 0.2, (K, F, F))
    if equal_rates:
        p['dom_del'] = p['dom_ins'] * (1 + 2e-5)
        p['main_del'] = p['main_ins'] * (1 + 2e-5)
    P = 5
    ts = np.exp(rng.uniform(-3, 1, P))
    names = ['main_ins', 'main_del', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates']

    def leaves(dev):
        d = {k: torch.tensor(np.asarray(p[k], float), dtype=torch.float64, device=dev, requires_grad=True)
             for k in names}
        d['t'] = torch.tensor(ts, dtype=torch.float64, device=dev, requires_grad=True)
        return d
    G = torch.as_tensor(rng.normal(size=(P, 2 + 5 * K * F, 2 + 5 * K * F)), dtype=torch.float64)
    a = leaves('cpu')
    ref = pm.build_nested_trans(a['main_ins'], a['main_del'], a['t'], a['dom_ins'], a['dom_del'],
                                a['dom_weights'], a['frag_weights'], a['ext_rates'])
    (ref * G).sum().backward()
    b = leaves('cuda')
    pro = _lib.MixDom2Prologue(dict(p))
    chi = api.MixDom2Chi.apply(pro, b['t'], b['main_ins'], b['main_del'], b['dom_ins'], b['dom_del'],
                               b['dom_weights'], b['frag_weights'], b['ext_rates'])
    torch.testing.assert_close(chi.cpu(), ref.detach(), rtol=1e-11, atol=1e-14)
    (chi * G.cuda()).sum().backward()
    for k in names + ['t']:
        want = a[k].grad
        scale = float(want.abs().max())
        torch.testing.assert_close(b[k].grad.cpu(), want, rtol=1e-9, atol=1e-10 * scale + 1e-14, msg=k)
