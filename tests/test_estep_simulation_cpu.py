"""E-step against simulation (the reference's test_estep_vs_simulation): pairs
drawn from the pair HMM itself -- a state path walked through chi from S to
E, characters drawn from the states' emission tables -- and the expected
transition counts of the float64 oracle's E-step, averaged over the pairs,
against the counts of the simulated paths (E[E[n | x, y]] = E[n]).  The
product equals the oracle to 1e-5 elsewhere; this pins the oracle's meaning
to the model rather than to the reference's code."""
import numpy as np
import pytest


def _simulate(rng, chi, st, EM, EI, ED, groups):
    """One pair: (x, y, realized transition counts)."""
    N = st.size
    e_idx = int(np.argmax(st == 4))
    n = np.zeros((N, N))
    x, y = [], []
    s = 0
    while True:
        k = int(rng.choice(N, p=chi[s] / chi[s].sum()))
        n[s, k] += 1
        if k == e_idx:
            return np.array(x, int), np.array(y, int), n
        g = groups[k]
        if st[k] == 1:
            J = EM[g][:20, :20] / EM[g][:20, :20].sum()
            ab = int(rng.choice(400, p=J.reshape(-1)))
            x.append(ab // 20)
            y.append(ab % 20)
        elif st[k] == 2:
            y.append(int(rng.choice(20, p=EI[g][:20] / EI[g][:20].sum())))
        elif st[k] == 3:
            x.append(int(rng.choice(20, p=ED[g][:20] / ED[g][:20].sum())))
        s = k


def _model(name, rng):
    from oracle import dp, models as om
    from pairhmm import synth
    from pairhmm import models as pm
    if name == 'tkf91':
        Q, pi, _ = synth.rand_Q_pi(rng)
        chi = om.tkf91_trans(0.05, 0.06, 0.6)
        st = np.array([0, 1, 2, 3, 4])
        groups = np.zeros(5, int)
        EM, EI, ED = dp.group_tables_tkf(om.transition_matrix(Q, 0.6), pi)
        return chi, st, groups, EM, EI, ED
    p = synth.mixdom2_params(rng, 2, 1, 2)
    t = 0.6
    chi = om.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'], p['dom_weights'],
                                p['frag_weights'], p['ext_rates'])
    st = pm.mixdom_state_types(2, 1)
    groups = pm.mixdom_state_groups(2, 1)
    csubs = om.build_class_subs(p['class_S_exch'], p['class_pis'], t)
    EM, EI, ED = dp.group_tables_per_class(csubs, p['class_pis'], p['classdist'])
    return chi, st, groups, EM, EI, ED


@pytest.mark.parametrize('name', ['tkf91', 'mixdom2'])
def test_expected_counts_match_simulation(name):
    from oracle import dp, models as om
    rng = np.random.default_rng(11 if name == 'tkf91' else 12)
    chi, st, groups, EM, EI, ED = _model(name, rng)
    lt = om.safe_log(chi)
    P = 400
    N = st.size
    exp_n = np.zeros((P, N, N))
    real_n = np.zeros((P, N, N))
    for p in range(P):
        # pairs longer than 30 residues in all are redrawn: the event depends on
        # (x, y) only, so E[E[n | x, y] | short] = E[n | short] still holds
        while True:
            x, y, n = _simulate(rng, chi, st, EM, EI, ED, groups)
            if x.size + y.size <= 30:
                break
        emit = dp.log_emission_table(st, groups, x, y, EM, EI, ED)
        _, _, e, _, _ = dp.forward_backward(lt, st, emit)
        exp_n[p], real_n[p] = e, n
    assert np.all(exp_n.sum(axis=(1, 2)) >= 1.0 - 1e-9)   # every path has at least S -> E
    # paired differences (each pair's expectation against its own path); a
    # floor on the error keeps transitions that were seldom drawn from
    # dominating on a handful of events
    d = exp_n - real_n
    se = d.std(axis=0) / np.sqrt(P) + 0.02 / np.sqrt(P)
    z = np.abs(d.mean(axis=0)) / se
    assert z.max() < 5.0, (z.max(), np.unravel_index(z.argmax(), z.shape))
    # totals: expected path length
    tot_e, tot_r = exp_n.sum(axis=(1, 2)), real_n.sum(axis=(1, 2))
    assert abs(tot_e.mean() - tot_r.mean()) < 5 * tot_r.std() / np.sqrt(P)
