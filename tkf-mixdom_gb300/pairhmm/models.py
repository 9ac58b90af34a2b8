"""Float64 torch builders of the pair-HMM parameters (the E-step prologue).

Differentiable restatements of the reference's builders, batched over
pairs where a per-pair evolutionary time t enters:
  * TKF BDI parameters alpha/beta/gamma/kappa with the L'Hopital branch
    (core/bdi.py:40-99);
  * TKF91 / TKF92 / MixFrag transition matrices (core/params.py:29-179);
  * the collapsed MixDom chi, N = 2 + 5KF (models/mixdom.py:52-77, 104-423);
  * per-class rate matrices and P_c(t) = expm(t Q_c) (train/vjp.py:463-510,
    core/ctmc.py:31-60);
  * per-group linear emission tables for the kernel: TKF (dp/hmm.py:628-670),
    MixDom2 per-class mixture (dp/hmm.py:673-783), MixDom1 per-domain
    (dp/hmm.py:786-851); index 20 is the wildcard with factor 1.
All tensors are float64; the DP consumes them cast to float32.
"""
from __future__ import annotations

import numpy as np
import torch

S, M, I, D, E = 0, 1, 2, 3, 4
EQUAL_RATE_THRESHOLD = 1e-4
F64 = torch.float64


def _t(x, device=None):
    if isinstance(x, torch.Tensor):
        return x.to(dtype=F64, device=device) if device is not None else x.to(F64)
    return torch.as_tensor(np.asarray(x, dtype=np.float64), dtype=F64, device=device)


# ---------------------------------------------------------------- BDI
def tkf_alpha(mu, t):
    return torch.exp(-mu * t)


def tkf_beta(lam, mu, t):
    """beta = lam(eta-alpha)/(mu eta - lam alpha); s/(1+s) when |1-kappa| < 1e-4."""
    s = mu * t
    eta = torch.exp(-lam * t)
    alpha = torch.exp(-s)
    numer = lam * (eta - alpha)
    denom = mu * eta - lam * alpha
    small = denom.abs() < 1e-30
    general = torch.where(small, torch.zeros_like(denom), numer / torch.where(small, torch.ones_like(denom), denom))
    limit = s / (1.0 + s)
    return torch.where((1.0 - lam / mu).abs() < EQUAL_RATE_THRESHOLD, limit, general)


def tkf_gamma(lam, mu, t):
    """gamma = 1 - mu beta / (lam (1-alpha)), L'Hopital limit at lam ~ mu."""
    s = mu * t
    alpha = tkf_alpha(mu, t)
    beta = tkf_beta(lam, mu, t)
    Phi = 1.0 - alpha
    general = torch.where(Phi.abs() < 1e-30, torch.zeros_like(Phi),
                          1.0 - mu * beta / (lam * Phi.clamp_min(1e-30)))
    phi = torch.where(s < 1e-10, 1.0 - s / 2.0, Phi / s.clamp_min(1e-30))
    limit = 1.0 - 1.0 / ((1.0 + s) * phi)
    return torch.where((1.0 - lam / mu).abs() < EQUAL_RATE_THRESHOLD, limit, general)


def tkf91_trans(lam, mu, t):
    """[..., 5, 5] TKF91 pair-HMM matrices (order S,M,I,D,E); lam, mu, t broadcast."""
    lam, mu, t = torch.broadcast_tensors(_t(lam), _t(mu), _t(t))
    a, b, g = tkf_alpha(mu, t), tkf_beta(lam, mu, t), tkf_gamma(lam, mu, t)
    k = lam / mu
    z = torch.zeros_like(a)
    row = torch.stack([z, (1 - b) * k * a, b, (1 - b) * k * (1 - a), (1 - b) * (1 - k)], dim=-1)
    rowD = torch.stack([z, (1 - g) * k * a, g, (1 - g) * k * (1 - a), (1 - g) * (1 - k)], dim=-1)
    zero = torch.zeros_like(row)
    return torch.stack([row, row, row, rowD, zero], dim=-2)


def tkf91_trans_cond(lam, mu, t):
    """[..., 5, 5] TKF91 matrices conditioned on the ancestor length
    (core/params.py:57-90): no kappa on M/D entries, no (1-kappa) on E."""
    lam, mu, t = torch.broadcast_tensors(_t(lam), _t(mu), _t(t))
    a, b, g = tkf_alpha(mu, t), tkf_beta(lam, mu, t), tkf_gamma(lam, mu, t)
    z = torch.zeros_like(a)
    row = torch.stack([z, (1 - b) * a, b, (1 - b) * (1 - a), 1 - b], dim=-1)
    rowD = torch.stack([z, (1 - g) * a, g, (1 - g) * (1 - a), 1 - g], dim=-1)
    zero = torch.zeros_like(row)
    return torch.stack([row, row, row, rowD, zero], dim=-2)


def tkf92_trans(lam, mu, t, ext):
    """TKF92: M/I/D rows scaled by (1-ext) with ext added on the diagonal."""
    t91 = tkf91_trans(lam, mu, t)
    ext = _t(ext)
    while ext.dim() < t91.dim() - 1:
        ext = ext.unsqueeze(-1)
    ext = ext[..., None]
    emit_rows = torch.tensor([0., 1., 1., 1., 0.], dtype=F64, device=t91.device)
    scale = 1.0 - ext * emit_rows[:, None]
    eye = torch.diag(emit_rows)
    return t91 * scale + ext * eye


def mixfrag_trans(lam, mu, t, exts, weights):
    """(3F+2)-state MixFrag matrix, order S, M_f, I_f, D_f, E (core/params.py:136-179)."""
    t91 = tkf91_trans(lam, mu, t)
    exts = _t(exts)
    w = _t(weights)
    F = exts.shape[0]
    n = 3 * F + 2
    typ = [M, I, D]
    rows = []
    # S row
    srow = [torch.zeros((), dtype=F64)]
    for ty in typ:
        srow += [w[g] * t91[S, ty] for g in range(F)]
    srow.append(t91[S, E])
    rows.append(torch.stack(srow))
    for sty in typ:
        for f in range(F):
            r = [torch.zeros((), dtype=F64)]
            for dty in typ:
                for g in range(F):
                    v = (1.0 - exts[f]) * w[g] * t91[sty, dty]
                    if sty == dty and f == g:
                        v = v + exts[f]
                    r.append(v)
            r.append((1.0 - exts[f]) * t91[sty, E])
            rows.append(torch.stack(r))
    rows.append(torch.zeros(n, dtype=F64))
    return torch.stack(rows)


def mixfrag_state_types(F):
    """Types of the (3F+2) MixFrag states S, M_1..M_F, I_1..I_F, D_1..D_F, E."""
    return np.array([S] + [M] * F + [I] * F + [D] * F + [E])


def mixfrag_trans_batch(lam, mu, t, exts, weights):
    """[B, 3F+2, 3F+2] MixFrag matrices for times t [B] (core/params.py:136-179,
    vectorised over t): entry (a, b) = row factor x TKF91[type a, type b] x
    column factor, with row factor 1 for S and (1 - ext_f) for an emitting
    state of fragment type f, column factor w_g for an emitting state of type
    g, 1 for E and 0 for S, plus ext_f on the diagonal of each emitting state;
    the E row is zero."""
    t91 = tkf91_trans(lam, mu, _t(t).reshape(-1))
    dev = t91.device
    exts = _t(exts, device=dev).reshape(-1)
    w = _t(weights, device=dev).reshape(-1)
    F = exts.shape[0]
    st = mixfrag_state_types(F)
    idx = torch.as_tensor(st, device=dev)
    base = t91[:, idx][:, :, idx]
    one, zero = torch.ones((), dtype=F64, device=dev), torch.zeros((), dtype=F64, device=dev)
    emit_f = [None] + list(range(F)) * 3 + [None]
    colw = torch.stack([zero] + [w[g] for g in emit_f[1:-1]] + [one])
    roww = torch.stack([one] + [1.0 - exts[f] for f in emit_f[1:-1]] + [zero])
    loop = torch.stack([zero] + [exts[f] for f in emit_f[1:-1]] + [zero])
    return roww[None, :, None] * base * colw[None, None, :] + torch.diag(loop)[None]


# ---------------------------------------------------------------- MixDom
_UV_EMIT = [M, I, D, I, D]
_UV_U = [M, M, M, I, D]
_UV_X = [M, I, D, I, D]
_IS_M = [True, True, True, False, False]
_MID = [M, I, D]


def mixdom_n_states(K, F):
    return 2 + 5 * K * F


def mixdom_state_types(K, F):
    body = np.tile(np.repeat(np.array(_UV_EMIT), F), K)
    return np.concatenate([[S, E], body]).astype(np.int8)


def mixdom_state_groups(K, F):
    """(d,f) group d*F+f of each body state (dp/hmm.py:719-729); 0 for SS/EE."""
    N = mixdom_n_states(K, F)
    g = np.zeros(N, dtype=np.int32)
    body = np.arange(N - 2)
    g[2:] = (body // (5 * F)) * F + (body % (5 * F)) % F
    return g


def mixdom1_state_groups(K, F):
    """Per-domain groups (dp/hmm.py:820-823)."""
    N = mixdom_n_states(K, F)
    g = np.zeros(N, dtype=np.int32)
    g[2:] = np.arange(N - 2) // (5 * F)
    return g


def _block_diag_batched(blocks):
    """Block-diagonal of a list of [..., a_i, a_i] tensors."""
    n = sum(b.shape[-1] for b in blocks)
    lead = blocks[0].shape[:-2]
    out = blocks[0].new_zeros(*lead, n, n)
    o = 0
    for b in blocks:
        k = b.shape[-1]
        out[..., o:o + k, o:o + k] = b
        o += k
    return out


def effective_trans_per_type(main_ins, main_del, t, dom_ins, dom_del, dom_w):
    """T_exit_k [..., K, 5, 5] and T_eff [..., 5, 5] (models/mixdom.py:104-214);
    t may carry a leading batch dimension."""
    t = _t(t)
    dom_ins, dom_del, dom_w = _t(dom_ins), _t(dom_del), _t(dom_w)
    K = dom_ins.shape[-1]
    tb = t[..., None]
    tau = tkf91_trans(_t(main_ins), _t(main_del), t)                       # [...,5,5]
    kap = dom_ins / dom_del                                                 # [K]
    bet = tkf_beta(dom_ins, dom_del, tb)                                    # [...,K]
    z_t = (1.0 - kap) * (1.0 - bet)
    z_0 = (1.0 - kap).expand_as(z_t)
    zeros5 = torch.zeros_like(tau[..., S, :])
    tau_rows = torch.stack([tau[..., S, :], tau[..., M, :], tau[..., I, :], tau[..., D, :], zeros5], dim=-2)
    tau_MID = tau_rows[..., :, _MID]                                        # [...,5,3]
    T_Nnull = (tau_MID[..., :, None, :] * dom_w[:, None]).reshape(*tau_MID.shape[:-1], 3 * K)
    nonnull = torch.stack([1.0 - z_t, kap.expand_as(z_t), kap.expand_as(z_t)], dim=-1)   # [...,K,3]
    null_prob = torch.stack([z_t, z_0, z_0], dim=-1)
    tauE = torch.stack([tau[..., M, E], tau[..., M, E], tau[..., D, E]], dim=-1)       # [...,3]
    lead = tau.shape[:-2]
    T_nullN = tau.new_zeros(*lead, K, 3, 5)
    for e in range(3):
        T_nullN[..., :, e, _MID[e]] = nonnull[..., :, e]
        T_nullN[..., :, e, E] = null_prob[..., :, e] * tauE[..., e, None]
    T_nullN = T_nullN.reshape(*lead, 3 * K, 5)
    tau_null_MID = torch.stack([tau[..., M, :], tau[..., M, :], tau[..., D, :]], dim=-2)[..., :, _MID]  # [...,3,3]
    z_flat = null_prob.reshape(*lead, 3 * K)
    ie = torch.arange(3 * K) % 3
    jk = torch.arange(3 * K) // 3
    T_nn = z_flat[..., :, None] * dom_w[jk][None, :] * tau_null_MID[..., ie[:, None], ie[None, :]]
    eye = torch.eye(3 * K, dtype=F64, device=tau.device)
    closure = torch.linalg.inv(eye - T_nn)
    closure_3d = closure.reshape(*lead, 3 * K, K, 3)
    T_nullN_3d = T_nullN.reshape(*lead, K, 3, 5)
    closure_exit = torch.einsum('...ike,...kev->...kiv', closure_3d, T_nullN_3d)
    T_exit_k = torch.einsum('...ui,...kiv->...kuv', T_Nnull, closure_exit)
    T_NN = torch.zeros_like(tau)
    T_NN[..., :, E] = tau_rows[..., :, E]
    return T_exit_k, T_NN + T_exit_k.sum(dim=-3)


def _nested_parts(main_ins, main_del, t, dom_ins, dom_del, dom_w, frag_w, ext_rates):
    """The factors of the collapsed MixDom chi (models/mixdom.py:252-423):
    exit_flat [..., nb] (exit_full), dest_flat [..., nb] (frag weight x
    entry factor), T_exit_k [..., K, 5, 5], the per-domain intra blocks
    [..., K, 5F, 5F], the SS row and EE column of the body, and the 5x5 T."""
    t = _t(t)
    dom_ins, dom_del, dom_w, frag_w = _t(dom_ins), _t(dom_del), _t(dom_w), _t(frag_w)
    ext = _t(ext_rates)
    if ext.dim() == 2:
        ext = torch.diag_embed(ext)
    K, F = frag_w.shape
    nb = K * 5 * F
    lead = t.shape
    T_exit_k, T = effective_trans_per_type(main_ins, main_del, t, dom_ins, dom_del, dom_w)
    tau_all = tkf91_trans(dom_ins, dom_del, t[..., None])                  # [...,K,5,5]
    kap = dom_ins / dom_del
    beta_d = (1.0 - tau_all[..., S, E]).clamp_min(1e-30)
    entry_M = tau_all[..., S, :][..., _UV_X] / beta_d[..., None]           # [...,K,5]
    isM = torch.tensor(_IS_M, device=tau_all.device)
    entry = torch.where(isM, entry_M, torch.ones_like(entry_M))
    exit_M = tau_all[..., :, E][..., _UV_X]
    exit_ID = (1.0 - kap)[:, None].expand_as(exit_M)
    exit_inner = torch.where(isM, exit_M, exit_ID)
    notext = 1.0 - ext.sum(dim=-1)                                          # [K,F]
    exit_full = notext[:, None, :] * exit_inner[..., :, :, None]            # [...,K,5,F]
    exit_flat = exit_full.reshape(*lead, nb)
    dest_flat = (frag_w[:, None, :] * entry[..., :, :, None]).reshape(*lead, nb)
    tau_MID_all = tau_all[..., _MID, :][..., _MID]                          # [...,K,3,3]
    nonext_M = torch.einsum('df,...dxy,dg->...dxfyg', notext, tau_MID_all, frag_w).reshape(*lead, K, 3 * F, 3 * F)
    ext_M = _block_diag_batched([ext, ext, ext])                            # [K,3F,3F]
    intra_M = nonext_M + ext_M
    nonext_I = (notext[:, :, None] * kap[:, None, None] * frag_w[:, None, :]).expand(*lead, K, F, F)
    intra_I = nonext_I + ext
    blocks = _block_diag_batched([intra_M, intra_I, intra_I])              # [...,K,bs,bs]
    ss_T = T_exit_k[..., :, S, :][..., _UV_U]                              # [...,K,5]
    ss_body = (ss_T[..., :, :, None] * frag_w[:, None, :] * entry[..., :, :, None]).reshape(*lead, nb)
    ee_body = (exit_full * T[..., _UV_U, E][..., None, :, None]).reshape(*lead, nb)
    return K, F, exit_flat, dest_flat, T_exit_k, blocks, ss_body, ee_body, T


def build_nested_trans(main_ins, main_del, t, dom_ins, dom_del, dom_w, frag_w, ext_rates):
    """Collapsed MixDom chi [..., N, N] (models/mixdom.py:252-423); t may be
    a [B] tensor of per-pair times."""
    K, F, exit_flat, dest_flat, T_exit_k, blocks, ss_body, ee_body, T = _nested_parts(
        main_ins, main_del, t, dom_ins, dom_del, dom_w, frag_w, ext_rates)
    lead = exit_flat.shape[:-1]
    nb = K * 5 * F
    N = 2 + nb
    bs = 5 * F
    T_kc = T_exit_k[..., :, _UV_U, :][..., _UV_U]                            # [...,K,5,5]
    d_idx = torch.arange(nb) // bs
    suv = torch.tensor(np.tile(np.repeat(np.arange(5), F), K))
    T_exp = T_kc[..., d_idx[None, :], suv[:, None], suv[None, :]]
    chi_inter = exit_flat[..., :, None] * T_exp * dest_flat[..., None, :]
    chi_intra = torch.zeros(*lead, nb, nb, dtype=F64, device=blocks.device)
    for k in range(K):
        chi_intra[..., k * bs:(k + 1) * bs, k * bs:(k + 1) * bs] = blocks[..., k, :, :]
    chi_body = chi_inter + chi_intra
    chi = torch.zeros(*lead, N, N, dtype=F64, device=chi_body.device)
    chi[..., 0, 1] = T[..., S, E]
    chi[..., 0, 2:] = ss_body
    chi[..., 2:, 1] = ee_body
    chi[..., 2:, 2:] = chi_body
    return chi


def nest_record_len(K, F):
    """Floats per pair of the nested chi record: exit [nb], cin [3][nb], intra [K][5F][5F]."""
    return 20 * K * F + 25 * K * F * F


def nested_record(main_ins, main_del, t, dom_ins, dom_del, dom_w, frag_w, ext_rates):
    """The collapsed MixDom chi in factored form, [..., R] float64 with
    R = nest_record_len(K, F), body states q = 0..nb-1 (state 2 + q, i.e.
    domain q // 5F, sub-state (q % 5F) // F, fragment q % F):
      exit[q]                      exit factor of source q (exit_full);
      cin[a][q], a = M, I, D       dest[q] * T_exit_k[d_q, a, U(q)];
      intra[d][i][j]               same-domain block without the inter part.
    For body states chi[2+s, 2+k] = exit[s] cin[U(s)][k] + [d_s = d_k] intra[d][s', k']
    (models/mixdom.py:343-394); the SS row and EE column stay in the dense chi."""
    K, F, exit_flat, dest_flat, T_exit_k, blocks, _, _, _ = _nested_parts(
        main_ins, main_del, t, dom_ins, dom_del, dom_w, frag_w, ext_rates)
    lead = exit_flat.shape[:-1]
    nb = K * 5 * F
    d_idx = torch.arange(nb) // (5 * F)
    u_of = torch.tensor(np.tile(np.repeat(np.asarray(_UV_U), F), K))       # main type of each body state
    cin = torch.stack([T_exit_k[..., d_idx, a, u_of] * dest_flat for a in (M, I, D)], dim=-2)   # [...,3,nb]
    return torch.cat([exit_flat, cin.reshape(*lead, 3 * nb), blocks.reshape(*lead, K * 25 * F * F)], dim=-1)


# ---------------------------------------------------------------- CTMC and emissions
def build_class_Q(S_exch, pis):
    """[C, A, A] rate matrices Q = S*pi off-diagonal, rows sum to 0 (train/vjp.py:463-476)."""
    S_exch, pis = _t(S_exch), _t(pis)
    Q = S_exch * pis[..., None, :]
    eye = torch.eye(Q.shape[-1], dtype=F64, device=Q.device)
    Q = Q * (1.0 - eye)
    return Q - torch.diag_embed(Q.sum(dim=-1))


def class_subs(S_exch, pis, t):
    """P_c(t) = expm(t Q_c) -> [..., C, A, A] for a scalar or [B] t."""
    Q = build_class_Q(S_exch, pis)
    t = _t(t, device=Q.device)
    return torch.linalg.matrix_exp(t[..., None, None, None] * Q)


def transition_matrix(Q, t):
    Q = _t(Q)
    t = _t(t, device=Q.device)
    return torch.linalg.matrix_exp(t[..., None, None] * Q)


def _pad21(x, lead_dims):
    """Append the wildcard row/col with factor 1."""
    if lead_dims == 1:
        return torch.cat([x, torch.ones_like(x[..., :1])], dim=-1)
    x = torch.cat([x, torch.ones_like(x[..., :1, :])], dim=-2)
    return torch.cat([x, torch.ones_like(x[..., :, :1])], dim=-1)


def tables_tkf(sub, pi):
    """G=1 tables of pair_hmm_emissions: (pi+1e-30)(P+1e-30) etc. -> EM [...,1,21,21], EI/ED [...,1,21]."""
    sub = _t(sub)
    pi = _t(pi, device=sub.device)
    lp = _pad21(pi + 1e-30, 1)
    ls = _pad21(sub + 1e-30, 2)
    lp = lp.expand(*sub.shape[:-2], 21)
    EM = lp[..., :, None] * ls
    return EM[..., None, :, :], lp[..., None, :], lp[..., None, :]


def tables_per_class(csubs, cpis, classdist):
    """MixDom2 tables: EM[g,a,b] = sum_c cd[g,c] max(pi_c[a],1e-30) max(P_c[a,b],1e-30),
    wildcard factor 1 (dp/hmm.py:673-783).  csubs [..., C, A, A]."""
    csubs = _t(csubs)
    cpis = _t(cpis, device=csubs.device)
    cd = _t(classdist, device=csubs.device)
    K, F, C = cd.shape
    cdg = cd.reshape(K * F, C)
    ls = _pad21(csubs.clamp_min(1e-30), 2)                           # [...,C,21,21]
    lp = _pad21(cpis.clamp_min(1e-30), 1)                            # [C,21]
    fM = lp[..., :, :, None] * ls                                    # [...,C,21,21]
    EM = torch.einsum('gc,...cab->...gab', cdg, fM)
    EI = torch.einsum('gc,ca->ga', cdg, lp)
    EI = EI.expand(*csubs.shape[:-3], *EI.shape)
    return EM, EI, EI


def tables_per_domain(subs, pis):
    """MixDom1 per-domain tables (dp/hmm.py:786-851): subs [..., K, A, A], pis [K, A]."""
    subs = _t(subs)
    pis = _t(pis, device=subs.device)
    ls = _pad21(subs.clamp_min(1e-30), 2)
    lp = _pad21(pis.clamp_min(1e-30), 1)
    EM = lp[..., :, :, None] * ls
    EI = lp.expand(*subs.shape[:-3], *lp.shape)
    return EM, EI, EI
