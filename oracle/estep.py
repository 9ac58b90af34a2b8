"""FP64 oracle: E-step outputs and custom-VJP cotangents (TEST INFRASTRUCTURE ONLY).

NumPy float64 restatement of the reference's E-step glue
(``python/tkfmixdom/jax/train/likelihood.py``) and of the emission-count
part of its MixDom2 custom VJP (``python/tkfmixdom/jax/train/vjp.py``).
Only the tests, ``smoke()`` and ``bench.py``'s CPU-baseline leg use it.
"""
from __future__ import annotations

import numpy as np

from . import models as om
from . import dp as odp
from .models import S, M, I, D, E


# ------------------------------------------------------------ model assembly
def tkf_model(model, params):
    """(chi, state_types, groups, EM, EI, ED) for 'tkf91' / 'tkf92'
    (train/likelihood.py:69-78)."""
    t = params['t']
    if model == 'tkf91':
        chi = om.tkf91_trans(params['ins_rate'], params['del_rate'], t)
    elif model == 'tkf92':
        chi = om.tkf92_trans(params['ins_rate'], params['del_rate'], t, params['ext'])
    else:
        raise ValueError(model)
    sub = om.transition_matrix(params['Q'], t)
    EM, EI, ED = odp.group_tables_tkf(sub, params['pi'])
    st = om.tkf_state_types()
    groups = np.zeros(5, dtype=np.int32)
    return chi, st, groups, EM, EI, ED, sub


def mixdom2_model(params):
    """(chi, state_types, groups, EM, EI, ED, class_subs) for MixDom2
    (train/likelihood.py:196-231)."""
    t = params['t']
    K = np.asarray(params['dom_ins']).shape[0]
    F = np.asarray(params['frag_weights']).shape[1]
    chi = om.build_nested_trans(params['main_ins'], params['main_del'], t,
                                params['dom_ins'], params['dom_del'],
                                params['dom_weights'], params['frag_weights'],
                                params['ext_rates'])
    cs = om.build_class_subs(params['class_S_exch'], params['class_pis'], t)
    EM, EI, ED = odp.group_tables_per_class(cs, params['class_pis'], params['classdist'])
    return (chi, om.mixdom_state_types(K, F), om.mixdom_state_groups(K, F),
            EM, EI, ED, cs)


# ------------------------------------------------------------ count tables
def char_count_tables(post, state_types, groups, x, y, G):
    """Per-group character-indexed posterior sums (the kernel's native
    emission-count output): cnt_M[g,a,b] = sum over cells with x_i=a, y_j=b
    of the M-type posteriors of group g; cnt_I[g,b] over y_j; cnt_D[g,a]
    over x_i.  Index 20 is the wildcard.  Row/col 0 never carry M/I/D mass
    of the wrong kind (dp/hmm.py:1241-1244)."""
    xg, yg = odp._grid_chars(x, y)
    st = np.asarray(state_types)
    cM = np.zeros((G, 21, 21))
    cI = np.zeros((G, 21))
    cD = np.zeros((G, 21))
    for k in range(st.size):
        g = groups[k]
        p = post[:, :, k]
        if st[k] == M:
            np.add.at(cM[g], (xg[1:, None], yg[None, 1:]), p[1:, 1:])
        elif st[k] == I:
            np.add.at(cI[g], yg[1:], p[:, 1:].sum(axis=0))
        elif st[k] == D:
            np.add.at(cD[g], xg[1:], p[1:, :].sum(axis=1))
    return cM, cI, cD


def observation_counts_2d(post, state_types, x, y, A):
    """match_anc_count / insert_count / delete_count
    (train/likelihood.py:962-1028); characters >= A are dropped
    (one_hot semantics)."""
    st = np.asarray(state_types)
    x = np.asarray(x, int)
    y = np.asarray(y, int)
    Lx, Ly = x.size, y.size
    Mp = post[:, :, st == M].sum(axis=2)[1:Lx + 1, 1:Ly + 1]
    Ip = post[:, :, st == I].sum(axis=2)[0:Lx + 1, 1:Ly + 1]
    Dp = post[:, :, st == D].sum(axis=2)[1:Lx + 1, 0:Ly + 1]
    out = {}
    for name, vals, chars in (('match_anc_count', Mp.sum(axis=1), x),
                              ('insert_count', Ip.sum(axis=0), y),
                              ('delete_count', Dp.sum(axis=1), x)):
        v = np.zeros(A)
        ok = chars < A
        np.add.at(v, chars[ok], vals[ok])
        out[name] = v
    return out


def match_pairs(post, state_types, x, y):
    """(a, b, w) for cells with M posterior > 1e-8 (train/likelihood.py:90-117)."""
    st = np.asarray(state_types)
    Lx, Ly = len(x), len(y)
    m = post[:, :, st == M].sum(axis=2)[1:Lx + 1, 1:Ly + 1]
    ii, jj = np.nonzero(m > 1e-8)
    xa = np.asarray(x, int)
    ya = np.asarray(y, int)
    return list(zip(xa[ii].tolist(), ya[jj].tolist(), m[ii, jj].tolist()))


# ------------------------------------------------------------ E-steps
def e_step(model, params, x, y):
    """TKF91/TKF92 E-step (train/likelihood.py:49-140):
    (LL, n_trans, {'match_pairs', 'pi_obs_counts'})."""
    if model == 'mixdom2':
        return e_step_mixdom2(params, x, y)
    chi, st, groups, EM, EI, ED, _ = tkf_model(model, params)
    emit = odp.log_emission_table(st, groups, x, y, EM, EI, ED)
    ll, post, n, _, _ = odp.forward_backward(om.safe_log(chi), st, emit)
    A = np.asarray(params['pi']).shape[0]
    ss = {'match_pairs': match_pairs(post, st, x, y),
          'pi_obs_counts': observation_counts_2d(post, st, x, y, A)}
    return ll, n, ss


def class_split(params, cM, cI, cD, wild_clamp=True):
    """MixDom2 per-class counts from the per-(d,f) character-indexed tables.

    The class posterior q[c | type, d, f, i, j] of train/likelihood.py:279-327
    depends on the cell only through its characters, so
        class_match[c,a,b] = sum_g cM[g,a,b] q_M[g,c,a,b]
    and likewise for insert/delete and classdist (likelihood.py:330-344).
    The per-class factors index class_pis/class_subs with the JAX gather
    clamp (character 20 reads index 19); one-hot over A=20 drops character 20
    from the character-indexed outputs."""
    cp = np.asarray(params['class_pis'], float)
    cd = np.asarray(params['classdist'], float)
    cs = om.build_class_subs(params['class_S_exch'], cp, params['t'])
    K, F, C = cd.shape
    A = cp.shape[1]
    cdg = cd.reshape(K * F, C)
    idx = np.minimum(np.arange(21), A - 1)
    fM = cp[:, idx][:, :, None] * cs[:, idx][:, :, idx]          # (C,21,21)
    fI = cp[:, idx]                                              # (C,21)
    jM = cdg[:, :, None, None] * fM[None]                        # (G,C,21,21)
    qM = jM / (jM.sum(axis=1, keepdims=True) + 1e-300)
    jI = cdg[:, :, None] * fI[None]
    qI = jI / (jI.sum(axis=1, keepdims=True) + 1e-300)
    wM = cM[:, None] * qM                                        # (G,C,21,21)
    wI = cI[:, None] * qI
    wD = cD[:, None] * qI
    return {
        'class_match_counts': wM.sum(axis=0)[:, :A, :A],
        'class_insert_counts': wI.sum(axis=0)[:, :A],
        'class_delete_counts': wD.sum(axis=0)[:, :A],
        'classdist_counts': (wM.sum(axis=(2, 3)) + wI.sum(axis=2)
                             + wD.sum(axis=2)).reshape(K, F, C),
    }


def e_step_mixdom2(params, x, y):
    """MixDom2 E-step (train/likelihood.py:143-373): LL, n_trans and the
    per-class sufficient-statistics dict including Holmes-Rubin class_W /
    class_U."""
    chi, st, groups, EM, EI, ED, cs = mixdom2_model(params)
    emit = odp.log_emission_table(st, groups, x, y, EM, EI, ED)
    ll, post, n, _, _ = odp.forward_backward(om.safe_log(chi), st, emit)
    G = EM.shape[0]
    cM, cI, cD = char_count_tables(post, st, groups, x, y, G)
    ss = class_split(params, cM, cI, cD)
    cp = np.asarray(params['class_pis'], float)
    W, U = [], []
    for c in range(cp.shape[0]):
        Qc = om.build_class_Q(params['class_S_exch'][c], cp[c])
        w, u = om.holmes_rubin_weighted_stats(Qc, cp[c], params['t'],
                                              ss['class_match_counts'][c])
        W.append(w)
        U.append(u)
    ss['class_W'] = np.stack(W)
    ss['class_U'] = np.stack(U)
    return ll, n, ss


def mixdom2_emission_counts(params, cM, cI, cD):
    """mc_c, V_c_linear, classdist_counts of ``_mixdom2_emission_counts``
    (train/vjp.py:513-625), from the per-(d,f) character tables.

    ratio = posterior / exp(emit) (emit the FB emission of the cell), so
    every term depends on the cell only through (g, a, b)."""
    cp = np.asarray(params['class_pis'], float)
    cd = np.asarray(params['classdist'], float)
    cs = om.build_class_subs(params['class_S_exch'], cp, params['t'])
    EM, EI, ED = odp.group_tables_per_class(cs, cp, cd)
    K, F, C = cd.shape
    A = cp.shape[1]
    cdg = cd.reshape(K * F, C)
    idx = np.minimum(np.arange(21), A - 1)
    fM = cp[:, idx][:, :, None] * cs[:, idx][:, :, idx]
    fI = cp[:, idx]
    rM = cM / EM                                                 # (G,21,21)
    rI = cI / EI
    rD = cD / ED
    wM = np.einsum('gab,gc,cab->cab', rM, cdg, fM)
    wI = np.einsum('gb,gc,cb->cb', rI, cdg, fI)
    wD = np.einsum('ga,gc,ca->ca', rD, cdg, fI)
    mc = wM[:, :A, :A]
    # match positions count by the ancestor character over every descendant
    # column, the wildcard included (vjp.py:601: one-hot over x only)
    V = wM[:, :A, :].sum(axis=2) + wI[:, :A] + wD[:, :A]
    sM = np.einsum('gab,cab->gc', rM, fM)
    sI = np.einsum('gb,cb->gc', rI, fI)
    sD = np.einsum('ga,ca->gc', rD, fI)
    cdc = (cdg * (sM + sI + sD)).reshape(K, F, C)
    return mc, V, cdc
