"""Reference-facing API of the 2D pair-HMM hot path.

Drop-in counterparts (same names, argument meaning, output layouts and dict
keys) of the reference's 2D pair-HMM entry points in
evoldoers/tkf-mixdom python/tkfmixdom/jax:

  forward_2d, backward_2d, forward_backward_2d   (dp/hmm.py:1775-1973)
  e_step, e_step_mixdom2, observed_ll           (train/likelihood.py:49-460)
  mixdom2_log_prob, tkf91_log_prob, tkf92_log_prob (train/vjp.py: custom VJPs)
  estep_batch_tkf92, estep_batch_tkf92_forward_only (train/tkf92_svi_bw.py:263-365)

plus the batched MixDom2 E-step ``estep_batch_mixdom2`` that replaces the
bucketed jit(vmap(...)) callers (train_pfam.py:1674-1741, 2672-2907).

All dynamic programming runs in the CUDA library (libpairhmm.so) through
the C ABI; this module only builds float64 model tables (pairhmm.models),
packs batches and runs float64 epilogues.  Numerical failure is reported the
reference's way: a log-likelihood of NEG_INF (-1e30).
"""
from __future__ import annotations

import functools
import math
import os

import numpy as np
import torch

from . import _lib
from . import autotune, graphs
from . import models as pm

NEG_INF = -1e30
S, M, I, D, E = pm.S, pm.M, pm.I, pm.D, pm.E


def _device():
    if not torch.cuda.is_available():
        raise _lib.PairHMMError('the pair-HMM library needs a CUDA device')
    return torch.device('cuda', torch.cuda.current_device())


# ---------------------------------------------------------------- padding semantics
def _make_geom_bins(base=4, max_bin=4096, mult=1.2):
    """Geometric bins of dp/hmm.py:43-63 (used only to shape padded outputs)."""
    bins = [int(base)]
    val = float(base)
    while val < max_bin:
        val *= mult
        b = int(round(val))
        if b > bins[-1]:
            bins.append(b)
    if bins[-1] < max_bin:
        bins.append(int(max_bin))
    return bins


_GEOM_BINS = [0, 1, 2, 3] + _make_geom_bins()


def pad_to_bin(n):
    """Padded size of dp/hmm.py:66-91 (TKFMIXDOM_MAX_PAD honoured)."""
    n = max(int(n), 1)
    cap = os.environ.get('TKFMIXDOM_MAX_PAD')
    if cap is not None:
        cap = int(cap)
        if n > cap:
            raise ValueError(f'_pad_to_bin: n={n} exceeds TKFMIXDOM_MAX_PAD={cap}')
        return max(min(((n + 31) // 32) * 32, cap), 1)
    for b in _GEOM_BINS:
        if b >= n:
            return b
    return int(2 ** math.ceil(math.log2(n)))


# ---------------------------------------------------------------- plans
@functools.lru_cache(maxsize=64)
def _plan(state_types_key, groups_key, G):
    return _lib.Plan(np.frombuffer(state_types_key, dtype=np.int8),
                     np.frombuffer(groups_key, dtype=np.int32), G)


def get_plan(state_types, groups, G):
    st = np.ascontiguousarray(np.asarray(state_types, dtype=np.int8))
    gr = np.ascontiguousarray(np.asarray(groups, dtype=np.int32))
    return _plan(st.tobytes(), gr.tobytes(), int(G))


def _chi_from_log(log_trans):
    lt = np.asarray(log_trans, dtype=np.float64)
    return np.where(lt > -1e29, np.exp(np.minimum(lt, 700.0)), 0.0)


def _groups_from_table(log_emit, state_types, x, y):
    """Recover per-group character tables from a (Lx+1, Ly+1, N) log
    emission table whose entries depend on the cell only through its
    characters (true of every emission builder of the reference), up to
    NEG_INF entries that cover every state of a type at a cell
    (mask_emissions_match_aligned, dp/hmm.py:1085-1117, and the banded
    recursions).  Returns (groups, EM, EI, ED, cell mask or None); the mask
    holds bit 0 / 1 / 2 where the M / I / D states may emit."""
    st = np.asarray(state_types)
    Lx, Ly = len(x), len(y)
    em = np.exp(np.asarray(log_emit, dtype=np.float64)[:Lx + 1, :Ly + 1])
    xg = np.concatenate([[0], np.asarray(x, int)])
    yg = np.concatenate([[0], np.asarray(y, int)])
    # per-type masks: a type is off at a cell when all its states emit 0 there
    on = {}
    for ty in (M, I, D):
        ks = np.nonzero(st == ty)[0]
        on[ty] = (em[:, :, ks] > 0).any(axis=2) if ks.size else np.ones((Lx + 1, Ly + 1), bool)
    groups = np.zeros(st.size, dtype=np.int32)
    tabs = []
    for k in range(st.size):
        if st[k] not in (M, I, D):
            continue
        TM = np.ones((21, 21))
        TI = np.ones(21)
        TD = np.ones(21)
        if st[k] == M:   # cells (i >= 1, j >= 1)
            v, use = em[1:, 1:, k], on[M][1:, 1:]
            ii, jj = np.nonzero(use)
            TM[xg[ii + 1], yg[jj + 1]] = v[ii, jj]
            got = TM[xg[1:, None], yg[None, 1:]]
        elif st[k] == I:   # cells (i >= 0, j >= 1)
            v, use = em[:, 1:, k], on[I][:, 1:]
            ii, jj = np.nonzero(use)
            TI[yg[jj + 1]] = v[ii, jj]
            got = np.broadcast_to(TI[yg[1:]][None, :], v.shape)
        else:   # cells (i >= 1, j >= 0)
            v, use = em[1:, :, k], on[D][1:, :]
            ii, jj = np.nonzero(use)
            TD[xg[ii + 1]] = v[ii, jj]
            got = np.broadcast_to(TD[xg[1:]][:, None], v.shape)
        if not np.allclose(got[use], v[use], rtol=1e-12, atol=0):
            raise NotImplementedError('log_emit_table entries must depend on the cell only through its '
                                      'characters, up to NEG_INF over all states of a type')
        # one group per state keeps the M/I/D tables of a group independent
        tabs.append((TM, TI, TD))
        groups[k] = len(tabs) - 1
    G = max(len(tabs), 1)
    EM = np.ones((G, 21, 21))
    EI = np.ones((G, 21))
    ED = np.ones((G, 21))
    for g, (TM, TI, TD) in enumerate(tabs):
        EM[g], EI[g], ED[g] = TM, TI, TD
    mask = (on[M].astype(np.uint8) | (on[I].astype(np.uint8) << 1) | (on[D].astype(np.uint8) << 2))
    # the lattice edges never use M (row/column 0), I (column 0) or D (row 0)
    need = np.ones((Lx + 1, Ly + 1), np.uint8) * 7
    need[0, :] &= ~np.uint8(5)
    need[:, 0] &= ~np.uint8(3)
    if np.all((mask & need) == need):
        return groups, EM, EI, ED, None
    mask[0, :] |= 5
    mask[:, 0] |= 3
    return groups, EM, EI, ED, mask


def _run_single_tables(chi, st, groups, EM, EI, ED, x, y, forward_only=False, cell_mask=None, beam=0.0):
    dev = _device()
    plan = get_plan(st, groups, EM.shape[0])
    b = _lib.make_batch([x], [y], np.asarray(chi)[None], np.asarray(EM)[None],
                        np.asarray(EI)[None], np.asarray(ED)[None], device=dev,
                        cell_masks=None if cell_mask is None else [cell_mask], beam_log_width=beam)
    out = _lib.estep_tables(plan, b, want_F=True, want_B=not forward_only,
                            want_post=not forward_only)
    Lx, Ly = len(x), len(y)
    N = len(st)
    res = {'ll': float(out['ll'][0]), 'status': int(out['status'][0]),
           'n_trans': out['n_trans'][0].cpu().numpy(),
           'cnt_M': out['cnt_M'][0].cpu().numpy(), 'cnt_I': out['cnt_I'][0].cpu().numpy(),
           'cnt_D': out['cnt_D'][0].cpu().numpy(),
           'F': out['log_F'].cpu().numpy().reshape(Lx + 1, Ly + 1, N)}
    if not forward_only:
        res['B'] = out['log_B'].cpu().numpy().reshape(Lx + 1, Ly + 1, N)
        res['post'] = out['post'].cpu().numpy().reshape(Lx + 1, Ly + 1, N)
    return res


def _tkf_tables(sub_matrix, pi):
    EM, EI, ED = pm.tables_tkf(sub_matrix, pi)
    return EM.numpy(), EI.numpy(), ED.numpy()


# ---------------------------------------------------------------- dp/hmm.py API
def forward_2d(log_trans, state_types, x_seq, y_seq, sub_matrix, pi):
    """(log P(x,y), F (Lx+1, Ly+1, N) log forward table) -- dp/hmm.py:1775-1801."""
    st = np.asarray(state_types)
    EM, EI, ED = _tkf_tables(sub_matrix, pi)
    r = _run_single_tables(_chi_from_log(log_trans), st, np.zeros(st.size, np.int32), EM, EI, ED,
                           np.asarray(x_seq), np.asarray(y_seq), forward_only=True)
    return r['ll'], r['F']


def backward_2d(log_trans, state_types, x_seq, y_seq, sub_matrix, pi):
    """B (Lx+1, Ly+1, N) log backward table -- dp/hmm.py:1804-1824.  Rows of
    states that are neither emitting nor the start state are NEG_INF."""
    st = np.asarray(state_types)
    EM, EI, ED = _tkf_tables(sub_matrix, pi)
    r = _run_single_tables(_chi_from_log(log_trans), st, np.zeros(st.size, np.int32), EM, EI, ED,
                           np.asarray(x_seq), np.asarray(y_seq))
    return r['B']


def forward_backward_2d(log_trans, state_types, x_seq, y_seq, sub_matrix, pi,
                        log_emit_table=None, real_Lx=None, real_Ly=None, forward_only=False):
    """(log_prob, posteriors, expected_trans) -- dp/hmm.py:1834-1973.

    Posteriors are returned at the reference's padded shape
    (pad_to_bin(Lx)+1, pad_to_bin(Ly)+1, N), zero outside the real region.
    real_Lx/real_Ly mark x_seq/y_seq as pre-padded."""
    st = np.asarray(state_types)
    x = np.asarray(x_seq)
    y = np.asarray(y_seq)
    Lx_arr, Ly_arr = x.shape[0], y.shape[0]
    Lx = Lx_arr if real_Lx is None else int(real_Lx)
    Ly = Ly_arr if real_Ly is None else int(real_Ly)
    xr, yr = x[:Lx], y[:Ly]
    mask = None
    if log_emit_table is not None:
        groups, EM, EI, ED, mask = _groups_from_table(log_emit_table, st, xr, yr)
    else:
        groups = np.zeros(st.size, np.int32)
        EM, EI, ED = _tkf_tables(sub_matrix, pi)
    r = _run_single_tables(_chi_from_log(log_trans), st, groups, EM, EI, ED, xr, yr,
                           forward_only=forward_only, cell_mask=mask)
    if forward_only:
        return r['ll']
    post = np.zeros((pad_to_bin(Lx_arr) + 1, pad_to_bin(Ly_arr) + 1, st.size))
    post[:Lx + 1, :Ly + 1] = r['post']
    return r['ll'], post, r['n_trans']


def _dense_log_table(state_types, groups, x_seq, y_seq, EM, EI, ED):
    """(Lx+1, Ly+1, N) log emission table from linear per-group tables: M
    states log EM[g][x_i][y_j], I log EI[g][y_j], D log ED[g][x_i], row and
    column 0 reading character 0, S / E states 0, log 0 as NEG_INF."""
    st = np.asarray(state_types)
    gr = np.asarray(groups, int)
    lg = lambda t: np.log(np.maximum(np.asarray(t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else t,
                                                np.float64), 1e-320))
    lM, lI, lD = lg(EM), lg(EI), lg(ED)
    xg = np.concatenate([[0], np.asarray(x_seq, int)])
    yg = np.concatenate([[0], np.asarray(y_seq, int)])
    out = np.zeros((xg.size, yg.size, st.size))
    for k in range(st.size):
        if st[k] == M:
            out[:, :, k] = lM[gr[k]][xg[:, None], yg[None, :]]
        elif st[k] == I:
            out[:, :, k] = lI[gr[k]][yg][None, :]
        elif st[k] == D:
            out[:, :, k] = lD[gr[k]][xg][:, None]
    out[out < -700.0] = NEG_INF
    return out


def pair_hmm_emissions(state_types, x_seq, y_seq, sub_matrix, pi):
    """dp/hmm.py:628-670: (Lx+1, Ly+1, N) log emissions log(pi+1e-30) +
    log(P+1e-30), wildcard 20 with probability 1, S/E states 0."""
    EM, EI, ED = pm.tables_tkf(pm._t(np.asarray(sub_matrix, np.float64)), pm._t(np.asarray(pi, np.float64)))
    return _dense_log_table(state_types, np.zeros(len(state_types), int), x_seq, y_seq, EM, EI, ED)


def pair_hmm_emissions_per_class(state_types, x_seq, y_seq, class_sub_matrices, class_pis, class_dist, n_dom,
                                 n_frag):
    """dp/hmm.py:673-783: the MixDom2 per-(domain, fragment) class-mixture
    log emissions, (Lx+1, Ly+1, N)."""
    EM, EI, ED = pm.tables_per_class(pm._t(np.asarray(class_sub_matrices, np.float64)),
                                     pm._t(np.asarray(class_pis, np.float64)),
                                     pm._t(np.asarray(class_dist, np.float64)))
    return _dense_log_table(state_types, pm.mixdom_state_groups(int(n_dom), int(n_frag)), x_seq, y_seq, EM, EI, ED)


def pair_hmm_emissions_per_domain(state_types, x_seq, y_seq, sub_matrices, pis, n_dom, n_frag):
    """dp/hmm.py:786-851: per-domain log emissions (domain d uses (pi_d, P_d),
    clamped at 1e-30), (Lx+1, Ly+1, N)."""
    EM, EI, ED = pm.tables_per_domain(pm._t(np.asarray(sub_matrices, np.float64)),
                                      pm._t(np.asarray(pis, np.float64)))
    N = len(state_types)
    groups = np.zeros(N, int)
    groups[2:] = np.arange(N - 2) // (5 * int(n_frag))
    return _dense_log_table(state_types, groups, x_seq, y_seq, EM, EI, ED)


def match_aligned_mask(Lx, Ly, match_i, match_j):
    """Cell mask of mask_emissions_match_aligned (dp/hmm.py:1085-1117): uint8
    (Lx+1, Ly+1) letting the M-type states emit only at the grid cells
    (mi+1, mj+1) of the training alignment (I and D everywhere)."""
    m = np.full((int(Lx) + 1, int(Ly) + 1), 6, np.uint8)
    m[np.asarray(match_i, int) + 1, np.asarray(match_j, int) + 1] |= 1
    return m


def mask_emissions_match_aligned(emit, state_types, match_positions_i, match_positions_j):
    """dp/hmm.py:1085-1117 on a host (Lx+1, Ly+1, N) log emission table: the
    M-type entries off the alignment's match cells (mi+1, mj+1) get NEG_INF
    added.  forward_backward_2d(..., log_emit_table=...) runs such a table on
    the cell-masked kernels; match_aligned_mask gives the mask directly."""
    em = np.array(emit, dtype=np.float64)
    allowed = np.zeros(em.shape[:2], bool)
    allowed[np.asarray(match_positions_i, int) + 1, np.asarray(match_positions_j, int) + 1] = True
    isM = np.asarray(state_types) == M
    em[:, :, isM] += np.where(allowed, 0.0, NEG_INF)[:, :, None]
    return em


def msa_to_band_center(msa_x_row, msa_y_row, Lx, gap_token=-1):
    """dp/hmm.py:2494-2525: band centres (Lx+1,) int32 from a guide alignment --
    for each i the j of the first point of the guide walk (0,0), (x_1, y_1), ...
    whose i reaches i (the last point where none does)."""
    has_x = np.asarray(msa_x_row).astype(np.int64) != gap_token
    has_y = np.asarray(msa_y_row).astype(np.int64) != gap_token
    gx = np.concatenate([[0], np.cumsum(has_x)])
    gy = np.concatenate([[0], np.cumsum(has_y)])
    idx = np.minimum(np.searchsorted(gx, np.arange(int(Lx) + 1), side='left'), gx.size - 1)
    return gy[idx].astype(np.int32)


def band_mask(Lx, Ly, band_center, band_width):
    """Cell mask of the banded recursions (dp/hmm.py:2104-2492): uint8
    (Lx+1, Ly+1), 7 where |j - c_i| <= W and 0 elsewhere, with
    W = pad_to_bin(band_width) as forward_backward_2d_banded pads it."""
    W = pad_to_bin(int(band_width))
    c = np.asarray(band_center, int)[:int(Lx) + 1]
    j = np.arange(int(Ly) + 1)
    return np.where(np.abs(j[None, :] - c[:, None]) <= W, 7, 0).astype(np.uint8)


def _to_band_layout(dense, band_center, W):
    Lx, Ly, N = dense.shape[0] - 1, dense.shape[1] - 1, dense.shape[2]
    Lp = pad_to_bin(Lx)
    c = np.full(Lp + 1, Ly)
    c[:Lx + 1] = np.asarray(band_center, int)[:Lx + 1]
    jj = c[:, None] - W + np.arange(2 * W + 1)[None, :]                 # (Lp+1, BW)
    ok = (jj >= 0) & (jj <= Ly) & (np.arange(Lp + 1)[:, None] <= Lx)
    out = np.zeros((Lp + 1, 2 * W + 1, N))
    ii, bb = np.nonzero(ok)
    out[ii, bb] = dense[ii, jj[ii, bb]]
    return out


def has_two_warp(plan):
    """Whether the plan's state space has two-warp stripe kernels (probed
    once: phmm_set_tuning refuses family 7 without them)."""
    v = getattr(plan, '_two_warp', None)
    if v is None:
        saved = plan.get_tuning()
        try:
            plan.set_tuning(**dict(saved, variant=7))
            v = True
        except _lib.PairHMMError:
            v = False
        finally:
            plan.set_tuning(**saved)
        plan._two_warp = v
    return v


def forward_backward_2d_banded(log_trans, state_types, x_seq, y_seq, sub_matrix, pi, band_center, band_width):
    """(log_prob, posteriors_bands, expected_trans) -- dp/hmm.py:2395-2491.

    The forward and backward recursions over the cells |j - c_i| <= W
    (W = pad_to_bin(band_width)); posteriors in the reference's band layout
    (pad_to_bin(Lx)+1, 2W+1, N), position (i, b) holding column c_i - W + b.
    Runs the cell-masked E-step (cells off the band emit nothing) through
    phmm_estep_band, whose stripes skip the anti-diagonal steps off their
    rows' band and which writes the band-layout posteriors on the device
    (O(L W) work); a state space without two-warp kernels takes the generic
    kernels' full tables instead.  For Lx off a padding bin the reference's
    own backward starts from a terminal band placed at row pad_to_bin(Lx)
    (dp/hmm.py:2337-2343) and its posteriors and counts are not those of the
    banded model; these are."""
    st = np.asarray(state_types)
    x, y = np.asarray(x_seq), np.asarray(y_seq)
    Lx, Ly = x.shape[0], y.shape[0]
    W = pad_to_bin(int(band_width))
    mask = band_mask(Lx, Ly, band_center, band_width)
    EM, EI, ED = _tkf_tables(sub_matrix, pi)
    chi = _chi_from_log(log_trans)
    groups = np.zeros(st.size, np.int32)
    plan = get_plan(st, groups, EM.shape[0])
    if not has_two_warp(plan):
        r = _run_single_tables(chi, st, groups, EM, EI, ED, x, y, cell_mask=mask)
        return r['ll'], _to_band_layout(r['post'], band_center, W), r['n_trans']
    b = _lib.make_batch([x], [y], np.asarray(chi)[None], np.asarray(EM)[None], np.asarray(EI)[None],
                        np.asarray(ED)[None], device=_device(), cell_masks=[mask])
    out = _lib.estep_band(plan, b, [np.asarray(band_center, int)[:Lx + 1]], W)
    post = np.zeros((pad_to_bin(Lx) + 1, 2 * W + 1, st.size))
    post[:Lx + 1] = out['post_band'].cpu().numpy()
    return float(out['ll'][0].item()), post, out['n_trans'][0].cpu().numpy()


def estep_batch_banded(log_trans, state_types, xs, ys, sub_matrix, pi, band_centers, band_width):
    """Batched forward_backward_2d_banded (the reference vmaps the single-pair
    call): one phmm_estep_band launch over every pair.  Returns (log_prob [P],
    posteriors_bands list of (pad_to_bin(Lx)+1, 2W+1, N), expected_trans
    [P, N, N]).  Needs a state space with two-warp kernels."""
    st = np.asarray(state_types)
    W = pad_to_bin(int(band_width))
    EM, EI, ED = _tkf_tables(sub_matrix, pi)
    plan = get_plan(st, np.zeros(st.size, np.int32), EM.shape[0])
    if not has_two_warp(plan):
        raise _lib.PairHMMError('estep_batch_banded: no two-warp kernels for this state space')
    xs = [np.asarray(x) for x in xs]
    ys = [np.asarray(y) for y in ys]
    masks = [band_mask(x.size, y.size, c, band_width) for x, y, c in zip(xs, ys, band_centers)]
    b = _lib.make_batch(xs, ys, np.asarray(_chi_from_log(log_trans))[None], np.asarray(EM)[None],
                        np.asarray(EI)[None], np.asarray(ED)[None], device=_device(), cell_masks=masks)
    out = _lib.estep_band(plan, b, [np.asarray(c, int)[:x.size + 1] for c, x in zip(band_centers, xs)], W)
    pb = out['post_band'].cpu().numpy()
    posts, r0 = [], 0
    for x in xs:
        p_ = np.zeros((pad_to_bin(x.size) + 1, 2 * W + 1, st.size))
        p_[:x.size + 1] = pb[r0:r0 + x.size + 1]
        posts.append(p_)
        r0 += x.size + 1
    return out['ll'].cpu().numpy(), posts, out['n_trans'].cpu().numpy()


def msa_to_envelope(x_len, y_len, msa_x_row, msa_y_row, band_width, gap_token=-1):
    """dp/hmm_beam.py:22-82: (x_len+1, y_len+1) bool envelope of the cells
    whose j lies within band_width of the y range of the guide points with i
    within band_width; (0, 0) and (x_len, y_len) always included."""
    pts = [(0, 0)]
    xi = yj = 0
    for a, b in zip(np.asarray(msa_x_row), np.asarray(msa_y_row)):
        xi += int(a) != gap_token
        yj += int(b) != gap_token
        pts.append((xi, yj))
    pts.append((x_len, y_len))
    pts = np.asarray(pts)
    i = np.arange(x_len + 1)
    near = np.abs(pts[None, :, 0] - i[:, None]) <= band_width               # (x_len+1, n_points)
    lo = np.where(near, pts[None, :, 1], y_len).min(axis=1)
    hi = np.where(near, pts[None, :, 1], 0).max(axis=1)
    j = np.arange(y_len + 1)
    env = (j[None, :] >= np.maximum(0, lo - band_width)[:, None]) & (j[None, :] <= np.minimum(y_len, hi + band_width)[:, None])
    env[0, 0] = True
    env[x_len, y_len] = True
    return env


def _beam_run(log_trans, state_types, x_seq, y_seq, sub_matrix, pi, beam_log_width, envelope, forward_only):
    st = np.asarray(state_types)
    x, y = np.asarray(x_seq), np.asarray(y_seq)
    w = float(beam_log_width)
    beam = w if np.isfinite(w) else 0.0
    if np.isfinite(w) and w <= 0:
        raise ValueError('beam_log_width must be positive (np.inf for no pruning)')
    mask = None
    if envelope is not None:
        env = np.asarray(envelope, bool)
        mask = np.where(env, 7, 0).astype(np.uint8)
        mask[0, 0] = 7                    # the start is never pruned (hmm_beam.py:122)
    # the beam module's emissions: log max(pi, 1e-30), log max(P, 1e-30)
    EM, EI, ED = pm.tables_per_domain(pm._t(np.asarray(sub_matrix, float))[None], pm._t(np.asarray(pi, float))[None])
    r = _run_single_tables(_chi_from_log(log_trans), st, np.zeros(st.size, np.int32), EM.numpy(), EI.numpy(),
                           ED.numpy(), x, y, forward_only=forward_only, cell_mask=mask, beam=beam)
    n_cells = int(np.count_nonzero(envelope)) - 1 if envelope is not None else (x.size + 1) * (y.size + 1) - 1
    return r, n_cells


def beam_forward_2d(log_trans, state_types, x_seq, y_seq, sub_matrix, pi, beam_log_width=np.inf, envelope=None):
    """(log_prob, F (Lx+1, Ly+1, N) log forward table, cells computed) --
    dp/hmm_beam.py:85-203: the forward restricted to the envelope with every
    state below its cell's maximum minus beam_log_width pruned."""
    r, n_cells = _beam_run(log_trans, state_types, x_seq, y_seq, sub_matrix, pi, beam_log_width, envelope, True)
    return r['ll'], r['F'], n_cells


def beam_forward_backward_2d(log_trans, state_types, x_seq, y_seq, sub_matrix, pi, beam_log_width=np.inf,
                             envelope=None):
    """(log_prob, posteriors (Lx+1, Ly+1, N), F) -- dp/hmm_beam.py:206-318:
    the pruned forward, the backward on the cells it left active, posteriors
    capped at 1 and 0 off the active cells."""
    r, _ = _beam_run(log_trans, state_types, x_seq, y_seq, sub_matrix, pi, beam_log_width, envelope, False)
    if not r['ll'] > -1e29:
        return r['ll'], np.zeros_like(r['F']), r['F']
    # the reference caps the posteriors at 1 and leaves the origin out of its
    # backward sweep (anti-diagonals Lx+Ly .. 1), so its posterior there is 0
    post = np.minimum(r['post'], 1.0)
    post[0, 0, :] = 0.0
    return r['ll'], post, r['F']


def iterative_beam_refinement(log_trans, state_types, x_seq, y_seq, sub_matrix, pi, beam_log_width=10.0,
                              initial_band=5, n_iterations=3, band_shrink=0.7):
    """dp/hmm_beam.py:321-394: beam forwards over a diagonal band that widens
    (x2) while the likelihood is empty and otherwise shrinks (x band_shrink,
    at least 2) around the previous run's active cells.  Returns (log_prob, F,
    envelope)."""
    Lx, Ly = len(x_seq), len(y_seq)

    def diagonal(band):
        c = np.rint(np.arange(Lx + 1) * Ly / max(Lx, 1)).astype(int)
        j = np.arange(Ly + 1)
        return (j[None, :] >= np.maximum(0, c - band)[:, None]) & (j[None, :] <= np.minimum(Ly, c + band)[:, None])
    band = initial_band
    env = diagonal(band)
    lp, F = -1e30, None
    for it in range(n_iterations):
        lp, F, _ = beam_forward_2d(log_trans, state_types, x_seq, y_seq, sub_matrix, pi, beam_log_width, env)
        if not lp > -1e30 + 100:
            band = int(band * 2)
            env = diagonal(band)
            continue
        if it < n_iterations - 1:
            active = np.any(F > -1e30 + 100, axis=2)
            nb = max(2, int(band * band_shrink))
            ii, jj = np.nonzero(active)
            acc = np.zeros((Lx + 2, Ly + 2), np.int64)   # 2D difference array of the dilated boxes
            np.add.at(acc, (np.maximum(ii - nb, 0), np.maximum(jj - nb, 0)), 1)
            np.add.at(acc, (np.minimum(ii + nb, Lx) + 1, np.maximum(jj - nb, 0)), -1)
            np.add.at(acc, (np.maximum(ii - nb, 0), np.minimum(jj + nb, Ly) + 1), -1)
            np.add.at(acc, (np.minimum(ii + nb, Lx) + 1, np.minimum(jj + nb, Ly) + 1), 1)
            env = acc.cumsum(axis=0).cumsum(axis=1)[:Lx + 1, :Ly + 1] > 0
            band = nb
    return lp, F, env


def beam_viterbi_2d(log_trans, state_types, x_seq, y_seq, sub_matrix, pi, envelope=None):
    """(log_prob, path as a list of (i, j, state)) -- dp/hmm_beam.py:397-490:
    the Viterbi recursion restricted to the envelope (a state whose cell or
    predecessor cell lies outside keeps NEG_INF and a pointer to the origin),
    emissions log max(pi, 1e-30) and log max(P, 1e-30)."""
    st = np.asarray(state_types)
    x, y = np.asarray(x_seq), np.asarray(y_seq)
    sub = np.asarray(sub_matrix, np.float64)
    p_ = np.asarray(pi, np.float64)
    A = p_.size
    lp = np.zeros(21)
    lp[:A] = np.log(np.maximum(p_, 1e-30))
    lM = np.zeros((21, 21))
    lM[:A, :A] = lp[:A, None] + np.log(np.maximum(sub, 1e-30))
    lM[:A, A:] = lp[:A, None]
    env = None
    if envelope is not None:
        env = [np.asarray(envelope, bool)]
        if env[0].shape != (x.size + 1, y.size + 1):
            raise ValueError('envelope must have shape (Lx+1, Ly+1)')
    ll, paths = _lib.viterbi(st, np.zeros(st.size, np.int32), 1, [x], [y], np.asarray(log_trans, np.float64)[None],
                             lM[None, None], lp[None, None], lp[None, None], device=_device(), envelopes=env)
    return float(ll[0]), [tuple(int(v) for v in row) for row in paths[0]]


_PRED_STEP = {M: (1, 1), I: (0, 1), D: (1, 0)}


def _draw_state(scores, rng):
    """A state index drawn with probability proportional to exp(scores) by
    rng.choice, or None when every score is within 100 of NEG_INF."""
    top = np.max(scores)
    if top <= NEG_INF + 100:
        return None
    w = np.exp(scores - top)
    return int(rng.choice(scores.size, p=w / w.sum()))


def beam_sample_traceback(log_trans, state_types, F, log_prob, x_seq, y_seq, sub_matrix, pi, rng, envelope=None):
    """Alignment path [(i, j, state), ...] from (0, 0, S) to (Lx, Ly, .) drawn
    from the posterior on a (beam-pruned) forward table -- dp/hmm_beam.py:493-563.

    The end state is drawn from F[Lx, Ly] + log_trans[:, E], then each
    predecessor from F[previous cell] + log_trans[:, current state], each draw
    one rng.choice on the normalised weights, so with the reference's
    numpy.random.RandomState and forward table the path is the same draw for
    draw.  The walk stops early (the origin is still appended) at a state that
    cannot step back from its cell, at a predecessor cell outside the
    envelope, or where every predecessor score is at NEG_INF; an empty list
    means the end cell itself is unreachable.  F is the (Lx+1, Ly+1, N) table
    of beam_forward_2d; log_prob, the residues, sub_matrix and pi are not
    read (the reference's signature)."""
    lt = np.asarray(log_trans)
    st = np.asarray(state_types)
    F = np.asarray(F)
    Lx, Ly = len(x_seq), len(y_seq)
    k = _draw_state(F[Lx, Ly, :] + lt[:, int(np.argmax(st == E))], rng)
    if k is None:
        return []
    i, j = Lx, Ly
    path = []
    while i > 0 or j > 0:
        path.append((i, j, k))
        di, dj = _PRED_STEP.get(int(st[k]), (i + 1, j + 1))
        if di > i or dj > j:
            break
        pi_, pj = i - di, j - dj
        if envelope is not None and not envelope[pi_, pj]:
            break
        prev = _draw_state(F[pi_, pj, :] + lt[:, k], rng)
        if prev is None:
            break
        i, j, k = pi_, pj, prev
    path.append((0, 0, int(S)))
    path.reverse()
    return path


def estep_batch_match_aligned(log_chi, state_types, xs, ys, match_is, match_js, sub_matrices, pis, n_dom, n_frag):
    """Batched match-aligned MixDom E-step (train_pfam.py:1744-1800,
    2946-2990: per-domain emissions, mask_emissions_match_aligned, the 2D
    forward-backward and the per-domain count reductions) in one cell-masked
    launch.

    log_chi [N,N] shared or [P,N,N] per pair; sub_matrices [K,A,A] shared or
    [P,K,A,A]; pis [K,A]; match_is / match_js: per-pair arrays of 0-based
    aligned positions.  Returns a dict of device tensors: log_prob [P],
    expected_trans [P,N,N], dom_match [P,K,20,20], dom_insert [P,K,20],
    dom_delete [P,K,20], agg_match [P,20,20], status [P]."""
    dev = _device()
    st = np.asarray(state_types)
    K, F = int(n_dom), int(n_frag)
    N = st.size
    groups = np.zeros(N, np.int32)
    groups[2:] = np.arange(N - 2) // (5 * F)                 # domain of each body state (dp/hmm.py:820-823)
    lc = np.asarray(log_chi.detach().cpu().numpy() if isinstance(log_chi, torch.Tensor) else log_chi, np.float64)
    chi = _chi_from_log(lc)
    if chi.ndim == 2:
        chi = chi[None]
    EM, EI, ED = pm.tables_per_domain(pm._t(sub_matrices), pm._t(pis))
    if EM.dim() == 4:
        EM, EI, ED = EM[None], EI[None], ED[None]
    masks = [match_aligned_mask(len(x), len(y), mi, mj) for x, y, mi, mj in zip(xs, ys, match_is, match_js)]
    b = _lib.make_batch(xs, ys, chi, EM, EI, ED, device=dev, cell_masks=masks)
    out = _lib.estep(get_plan(st, groups, K), b)
    dm = out['cnt_M'][:, :, :20, :20]
    return {'log_prob': out['ll'], 'expected_trans': out['n_trans'], 'dom_match': dm,
            'dom_insert': out['cnt_I'][:, :, :20], 'dom_delete': out['cnt_D'][:, :, :20],
            'agg_match': dm.sum(dim=1), 'status': out['status']}


# ---------------------------------------------------------------- E-steps
def _tkf_model(model, params):
    t = params['t']
    if model in ('tkf91',):
        chi = pm.tkf91_trans(params['ins_rate'], params['del_rate'], t)
    elif model == 'tkf92':
        chi = pm.tkf92_trans(params['ins_rate'], params['del_rate'], t, params['ext'])
    else:
        raise ValueError(f'Unknown model: {model}')
    sub = pm.transition_matrix(params['Q'], t)
    EM, EI, ED = pm.tables_tkf(sub, params['pi'])
    st = np.array([S, M, I, D, E], np.int8)
    return chi.numpy(), st, np.zeros(5, np.int32), EM.numpy(), EI.numpy(), ED.numpy()


def _mixdom1_model(params):
    t = params['t']
    K = len(params['dom_ins'])
    F = np.asarray(params['frag_weights']).shape[1]
    chi = pm.build_nested_trans(params['main_ins'], params['main_del'], t, params['dom_ins'],
                                params['dom_del'], params['dom_weights'], params['frag_weights'],
                                params['ext_rates'])
    sub = pm.transition_matrix(params['Q'], t)
    EM, EI, ED = pm.tables_tkf(sub, params['pi'])
    return (chi.numpy(), pm.mixdom_state_types(K, F), np.zeros(pm.mixdom_n_states(K, F), np.int32),
            EM.numpy(), EI.numpy(), ED.numpy())


def e_step(model, params, x, y):
    """E-step (train/likelihood.py:49-140): (LL, n_trans, ss) with
    ss = {'match_pairs': [(a, b, w)], 'pi_obs_counts': {...}} for
    tkf91/tkf92/mixdom; dispatches to e_step_mixdom2 for 'mixdom2'."""
    if model == 'mixdom2':
        return e_step_mixdom2(params, x, y)
    if model == 'mixdom':
        chi, st, groups, EM, EI, ED = _mixdom1_model(params)
    else:
        chi, st, groups, EM, EI, ED = _tkf_model(model, params)
    x = np.asarray(x)
    y = np.asarray(y)
    r = _run_single_tables(chi, st, groups, EM, EI, ED, x, y)
    post = r['post']
    Lx, Ly = len(x), len(y)
    mpost = post[1:, 1:, st == M].sum(axis=2)
    ii, jj = np.nonzero(mpost > 1e-8)
    match_pairs = list(zip(x[ii].astype(int).tolist(), y[jj].astype(int).tolist(),
                           mpost[ii, jj].astype(np.float64).tolist()))
    A = int(np.asarray(params['pi']).shape[0])
    cM, cI, cD = r['cnt_M'].sum(axis=0), r['cnt_I'].sum(axis=0), r['cnt_D'].sum(axis=0)
    pi_obs = {'match_anc_count': cM[:A, :].sum(axis=1), 'insert_count': cI[:A].copy(),
              'delete_count': cD[:A].copy()}
    return r['ll'], r['n_trans'], {'match_pairs': match_pairs, 'pi_obs_counts': pi_obs}


def class_split(params, cM, cI, cD, csubs=None):
    """Per-class MixDom2 counts from per-(d,f) character tables
    (train/likelihood.py:279-344), float64 torch, batched over leading dims.

    The class posterior q[c | type, d, f, i, j] depends on the cell only
    through its characters, so the lattice-sized joints of the reference
    collapse to 21x21 character tables.  Character 20 (wildcard) reads the
    class factors at index A-1 (JAX gather clamp) and is dropped from the
    character-indexed outputs (one-hot over A)."""
    cp = pm._t(params['class_pis'], device=cM.device)
    cd = pm._t(params['classdist'], device=cM.device)
    if csubs is None:
        csubs = pm.class_subs(params['class_S_exch'], cp, params['t']).to(cM.device)
    K, F, C = cd.shape
    A = cp.shape[1]
    cdg = cd.reshape(K * F, C)
    idx = torch.clamp(torch.arange(21, device=cM.device), max=A - 1)
    fM = cp[:, idx][:, :, None] * csubs[..., :, idx, :][..., idx]            # [...,C,21,21]
    fI = cp[:, idx]                                                         # [C,21]
    jM = cdg[:, :, None, None] * fM[..., None, :, :, :]                     # [...,G,C,21,21]
    qM = jM / (jM.sum(dim=-3, keepdim=True) + 1e-300)
    jI = cdg[:, :, None] * fI[None]
    qI = jI / (jI.sum(dim=-2, keepdim=True) + 1e-300)                       # [G,C,21]
    wM = cM[..., :, None, :, :] * qM
    wI = cI[..., :, None, :] * qI
    wD = cD[..., :, None, :] * qI
    return {
        'class_match_counts': wM.sum(dim=-4)[..., :A, :A],
        'class_insert_counts': wI.sum(dim=-3)[..., :A],
        'class_delete_counts': wD.sum(dim=-3)[..., :A],
        'classdist_counts': (wM.sum(dim=(-2, -1)) + wI.sum(dim=-1) + wD.sum(dim=-1)).reshape(
            *wM.shape[:-4], K, F, C),
    }


def holmes_rubin_weighted_stats(Q, pi, t, mc):
    """W[i], U[i,j] (core/ctmc.py:173-230, 285-326) of one (Q, pi, t) and one
    [A, A] match-count grid, float64 host tensors, through phmm_holmes_rubin."""
    Qh = pm._t(Q).cpu().numpy()
    pih = pm._t(pi).cpu().numpy()
    dev = _device()
    mcd = pm._t(mc).to(dev).reshape(1, 1, *Qh.shape)
    W, U = _lib.holmes_rubin(Qh, pih, torch.tensor([float(t)], dtype=torch.float64, device=dev), mcd)
    return W[0, 0].cpu(), U[0, 0].cpu()


def holmes_rubin_batch(class_S_exch, class_pis, ts, class_match_counts, out=None):
    """Batched Holmes-Rubin statistics (core/ctmc.py:173-230, 285-326) for
    per-pair times ts [P] and per-pair per-class match counts [P, C, A, A]:
    W [P, C, A] (expected dwell times) and U [P, C, A, A] (expected
    substitutions, zero diagonal), float64 on the counts' device, by the
    phmm_holmes_rubin kernel (one CTA per pair and class contracting the
    eigendecomposition of the symmetrised class rate matrix; no A^4 endpoint
    tensor)."""
    mc = class_match_counts if isinstance(class_match_counts, torch.Tensor) else torch.as_tensor(
        np.asarray(class_match_counts))
    S = np.asarray(pm._t(class_S_exch).cpu().numpy(), np.float64)
    pis = np.asarray(pm._t(class_pis).cpu().numpy(), np.float64)
    Q = S * pis[:, None, :]
    for c in range(Q.shape[0]):
        np.fill_diagonal(Q[c], 0.0)
        np.fill_diagonal(Q[c], -Q[c].sum(axis=1))
    t = ts if isinstance(ts, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(np.asarray(ts, np.float64)))
    return _lib.holmes_rubin(Q, pis, t.to(mc.device), mc, out=out)


def _mixdom2_tables(params, ts, device):
    K = len(params['dom_ins'])
    F = np.asarray(params['frag_weights']).shape[1]
    ts = pm._t(ts, device=device)
    chi = pm.build_nested_trans(params['main_ins'], params['main_del'], ts.cpu(), params['dom_ins'],
                                params['dom_del'], params['dom_weights'], params['frag_weights'],
                                params['ext_rates']).to(device)
    csubs = pm.class_subs(pm._t(params['class_S_exch'], device), pm._t(params['class_pis'], device), ts)
    EM, EI, ED = pm.tables_per_class(csubs, pm._t(params['class_pis'], device),
                                     pm._t(params['classdist'], device))
    return K, F, chi, csubs, EM, EI, ED


def _mixdom2_nest(params, ts, device):
    """The factored transitions of _mixdom2_tables' chi, float32 [P, R] on
    `device` (models.nested_record; phmm_batch.nest)."""
    rec = pm.nested_record(params['main_ins'], params['main_del'], pm._t(ts), params['dom_ins'],
                           params['dom_del'], params['dom_weights'], params['frag_weights'], params['ext_rates'])
    return rec.to(device=device, dtype=torch.float32).contiguous()


def to_host(result):
    """A result dict of device tensors as host numpy arrays, copied with one
    synchronisation (asynchronous copies into reused pinned memory)."""
    return _lib.to_host(result)


def forward_backward_1d_batch(log_trans, log_emissions, seq_lengths, init_state=S, final_state=E):
    """Batched forward_backward_1d_padded (dp/hmm.py:471-607) on the device.

    log_trans: [N, N] or per pair [B, N, N] log transitions; log_emissions
    [B, L_pad, N] with the real columns first; seq_lengths [B].  Returns
    (log_prob [B], posteriors [B, L_pad, N] (0 at padded columns),
    expected_trans [B, N, N]) as float64 device tensors."""
    dev = _device()
    le = torch.as_tensor(np.asarray(log_emissions) if not isinstance(log_emissions, torch.Tensor) else log_emissions)
    le = le.to(device=dev, dtype=torch.float64)
    B, Lp, N = le.shape
    lens = np.asarray(seq_lengths, np.int64).reshape(-1)
    lt = torch.as_tensor(np.asarray(log_trans) if not isinstance(log_trans, torch.Tensor) else log_trans)
    lt = lt.to(device=dev, dtype=torch.float64)
    chi = torch.where(lt > -1e29, torch.exp(lt), torch.zeros_like(lt)).to(torch.float32).contiguous()
    mask = torch.arange(Lp, device=dev)[None, :] < torch.as_tensor(lens, device=dev)[:, None]
    rows = torch.where(le > -1e29, torch.exp(le), torch.zeros_like(le)).to(torch.float32)[mask].contiguous()
    off = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
    ll, nt, post, _ = _lib.fb1d(N, lens, off, rows if rows.numel() else torch.zeros(1, N, device=dev), chi,
                                chi.dim() == 3, init_state, final_state, posteriors=True)
    posteriors = torch.zeros(B, Lp, N, dtype=torch.float64, device=dev)
    if rows.numel():
        posteriors[mask] = post[:int(lens.sum())].to(torch.float64)
    return ll, posteriors, nt


def estep_1d_mixdom2(params, cols, ancs, descs, ts, with_posteriors=False):
    """Alignment-conditioned MixDom2 E-step (the 1D path of the reference's
    training loop, dp/hmm.py:471-607 with pair_hmm_emissions_constrained_per_class,
    dp/hmm.py:981-1082), batched over pairs: cols[p] the per-column state
    types (1 M, 2 I, 3 D) of pair p's alignment, ancs[p] / descs[p] its
    ancestor / descendant characters per column (used at M and D / M and I
    columns; 20 = wildcard), ts[p] its time.  Returns device tensors log_p
    [P], n_trans [P, N, N], status [P] and, with with_posteriors, posteriors
    as a list of [L_p, N] float32."""
    dev = _device()
    pro = _lib.MixDom2Prologue(params)
    chi, EM, EI, ED, _ = pro(ts, device=dev)
    K, F = pro.K, pro.F
    st = pm.mixdom_state_types(K, F)
    gr = pm.mixdom_state_groups(K, F)
    lens = np.array([len(c) for c in cols], np.int64)
    off = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
    cat = lambda xs: torch.from_numpy(np.concatenate([np.asarray(x, np.uint8).reshape(-1) for x in xs])
                                      if lens.sum() else np.zeros(1, np.uint8)).to(dev)
    emit, st1 = _lib.fb1d_emissions(st, gr, K * F, lens, off, cat(cols), cat(ancs), cat(descs), EM, EI, ED, True)
    ll, nt, post, st2 = _lib.fb1d(len(st), lens, off, emit, chi, True, 0, 1, posteriors=with_posteriors)
    res = {'log_p': ll, 'n_trans': nt, 'status': st1 | st2}
    if with_posteriors:
        res['posteriors'] = [post[o:o + n] for o, n in zip(off, lens)]
    return res


class ConstrainedLogLik(torch.autograd.Function):
    """Sum of per-alignment 1D log-likelihoods (phmm_fb1d) with the
    score-identity adjoint: dLL/dchi = n_trans/chi, dLL/dEM = cnt_M/EM (and I,
    D alike), the character counts summed from the column posteriors -- the
    gradient train/vjp.py:1325-1437 returns for the constrained DP."""

    @staticmethod
    def forward(ctx, chi, EM, EI, ED, st, gr, cols, ancs, descs):
        dev = chi.device
        P = len(cols)
        N, G = len(st), EM.shape[1]
        lens = np.array([len(c) for c in cols], np.int64)
        off = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
        cat = lambda xs: (np.concatenate([np.asarray(x, np.int64).reshape(-1) for x in xs])
                          if lens.sum() else np.zeros(1, np.int64))
        c_all, a_all, d_all = cat(cols), cat(ancs), cat(descs)
        to_u8 = lambda a: torch.from_numpy(np.clip(a, 0, 255).astype(np.uint8)).to(dev)
        f32 = lambda v: v.detach().to(torch.float32).contiguous()
        per_pair = EM.shape[0] == P
        emit, st1 = _lib.fb1d_emissions(st, gr, G, lens, off, to_u8(c_all), to_u8(a_all), to_u8(d_all),
                                        f32(EM), f32(EI), f32(ED), per_pair)
        ll, nt, post, st2 = _lib.fb1d(N, lens, off, emit, f32(chi), chi.shape[0] == P and chi.dim() == 3, 0, 1,
                                      posteriors=True)
        # character counts per pair from the column posteriors
        ncol = int(lens.sum())
        pair_of = torch.as_tensor(np.repeat(np.arange(P), lens), device=dev)
        cM = torch.zeros(P * G * 441, dtype=torch.float64, device=dev)
        cI = torch.zeros(P * G * 21, dtype=torch.float64, device=dev)
        cD = torch.zeros(P * G * 21, dtype=torch.float64, device=dev)
        if ncol:
            pst = post[:ncol].to(torch.float64)
            c_t = torch.as_tensor(c_all[:ncol], device=dev)
            a_t = torch.as_tensor(np.minimum(a_all[:ncol], 20), device=dev)
            d_t = torch.as_tensor(np.minimum(d_all[:ncol], 20), device=dev)
            st_t = torch.as_tensor(np.asarray(st, np.int64), device=dev)
            gr_t = torch.as_tensor(np.asarray(gr, np.int64), device=dev)
            for typ, out, idx_fn in ((1, cM, lambda g: (pair_of[:, None] * G + g) * 441 + a_t[:, None] * 21
                                      + d_t[:, None]),
                                     (2, cI, lambda g: (pair_of[:, None] * G + g) * 21 + d_t[:, None]),
                                     (3, cD, lambda g: (pair_of[:, None] * G + g) * 21 + a_t[:, None])):
                sel = st_t == typ
                if not bool(sel.any()):
                    continue
                w = pst[:, sel] * (c_t == typ)[:, None]
                out.index_add_(0, idx_fn(gr_t[sel][None, :]).reshape(-1), w.reshape(-1))
        cM, cI, cD = cM.view(P, G, 21, 21), cI.view(P, G, 21), cD.view(P, G, 21)
        ctx.save_for_backward(chi, EM, EI, ED, nt, cM, cI, cD)
        ctx.status = st1 | st2
        return ll

    @staticmethod
    def backward(ctx, g):
        chi, EM, EI, ED, n, cM, cI, cD = ctx.saved_tensors
        gw = g.to(torch.float64)

        def ratio(cnt, tab):
            per_pair = tab.shape[0] == cnt.shape[0]
            r = torch.where(tab > 0, cnt / torch.where(tab > 0, tab, torch.ones_like(tab)), torch.zeros_like(cnt))
            r = r * gw.reshape((-1,) + (1,) * (cnt.dim() - 1))
            return (r if per_pair else r.sum(dim=0, keepdim=True)).to(tab.dtype)
        return (ratio(n, chi), ratio(cM, EM), ratio(cI, EI), ratio(cD, ED), None, None, None, None, None)


def mixdom2_constrained_log_prob(main_ins_rate, main_del_rate, t, dom_ins_rates, dom_del_rates, dom_weights,
                                 frag_weights, ext_rates, class_S_exch, class_pis, classdist, state_seq,
                                 anc_chars, desc_chars, real_L=None):
    """1D log P(x, y, A | params) under MixDom2 along fixed alignments
    (train/vjp.py:1193-1229), differentiable in every parameter tensor.
    state_seq / anc_chars / desc_chars: one alignment (arrays; real_L its
    length) or lists of alignments, in which case t is [P] and the result [P]."""
    dev = _device()
    batched = isinstance(state_seq, (list, tuple))
    if batched:
        cols, ancs, descs = list(state_seq), list(anc_chars), list(desc_chars)
    else:
        Lr = len(state_seq) if real_L is None else int(real_L)
        cols, ancs, descs = [np.asarray(state_seq)[:Lr]], [np.asarray(anc_chars)[:Lr]], [np.asarray(desc_chars)[:Lr]]
    tt = pm._t(t, device=dev).reshape(-1)
    f = lambda v: pm._t(v, device=dev)
    K, F = f(frag_weights).shape
    if K * F <= 12 and f(class_pis).shape[-1] == 20:
        pro = _lib.MixDom2Prologue({
            'main_ins': main_ins_rate, 'main_del': main_del_rate, 'dom_ins': dom_ins_rates,
            'dom_del': dom_del_rates, 'dom_weights': dom_weights, 'frag_weights': frag_weights,
            'ext_rates': ext_rates, 'class_pis': class_pis, 'class_S_exch': class_S_exch,
            'classdist': classdist})
        chi = MixDom2Chi.apply(pro, tt, f(main_ins_rate), f(main_del_rate), f(dom_ins_rates), f(dom_del_rates),
                               f(dom_weights), f(frag_weights), f(ext_rates))
    else:
        chi = pm.build_nested_trans(f(main_ins_rate), f(main_del_rate), tt, f(dom_ins_rates),
                                    f(dom_del_rates), f(dom_weights), f(frag_weights), f(ext_rates))
    csubs = pm.class_subs(f(class_S_exch), f(class_pis), tt)
    EM, EI, ED = pm.tables_per_class(csubs, f(class_pis), f(classdist))
    if EI.dim() == 2:
        EI, ED = EI.unsqueeze(0), ED.unsqueeze(0)
    st = pm.mixdom_state_types(K, F)
    gr = pm.mixdom_state_groups(K, F)
    ll = ConstrainedLogLik.apply(chi, EM, EI, ED, st, gr, cols, ancs, descs)
    return ll if batched else ll[0]


def _log_tkf_tables(sub_matrix, pi):
    """The log emission terms of _pair_hmm_emission (dp/hmm.py:617-625) as per-group
    tables: M[a][b] = log(pi_a + 1e-30) + log(P_ab + 1e-30), I/D[a] = log(pi_a + 1e-30),
    index 20 (wildcard) log 1."""
    sub = np.asarray(sub_matrix, np.float64)
    pi_ = np.asarray(pi, np.float64)
    A = pi_.size
    lp = np.zeros(21)
    lp[:A] = np.log(pi_ + 1e-30)
    lM = np.zeros((21, 21))
    lM[:A, :A] = np.log(pi_ + 1e-30)[:, None] + np.log(sub + 1e-30)
    lM[:A, A:] = np.log(pi_ + 1e-30)[:, None]
    return lM[None, None], lp[None, None], lp[None, None]


def viterbi_2d_batch(log_trans, state_types, xs, ys, sub_matrix, pi):
    """Batched viterbi_2d (dp/hmm.py:1976-2040) on the device: per pair the
    log-probability of the best path and the path as (i, j, state) triples
    from (0, 0, S) to (Lx, Ly, final state)."""
    lt = np.asarray(log_trans, np.float64)
    st = np.asarray(state_types)
    lM, lI, lD = _log_tkf_tables(sub_matrix, pi)
    ll, paths = _lib.viterbi(st, np.zeros(st.size, np.int32), 1, xs, ys, lt[None], lM, lI, lD,
                             device=_device())
    return ll, [[tuple(int(v) for v in row) for row in pth] for pth in paths]


def viterbi_2d(log_trans, state_types, x_seq, y_seq, sub_matrix, pi):
    """viterbi_2d (dp/hmm.py:1976-2040): (log_prob, path as a list of (i, j, state))."""
    ll, paths = viterbi_2d_batch(log_trans, state_types, [np.asarray(x_seq)], [np.asarray(y_seq)],
                                 sub_matrix, pi)
    return float(ll[0]), paths[0]


def _seed_of(rng_key):
    """A 64-bit seed from an int or an array of integers (e.g. a two-word
    PRNG key), the words packed little end first."""
    if isinstance(rng_key, (int, np.integer)):
        return int(rng_key) & 0xFFFFFFFFFFFFFFFF
    words = np.asarray(rng_key).astype(np.uint64).reshape(-1)
    seed = 0
    for k, w in enumerate(words[:2]):
        seed |= (int(w) & 0xFFFFFFFF) << (32 * k)
    return seed


def sample_traceback_2d_batch(log_trans, state_types, xs, ys, sub_matrix, pi, n_samples, seed=0):
    """Batched stochastic forward traceback (dp/hmm.py:2043-2101) on the
    device: (log_prob [P] float64, paths: per pair a list of n_samples paths,
    each a list of (i, j, state) from (0, 0, S) to (Lx, Ly, final state)),
    drawn from the posterior over alignments.  The same seed gives the same
    paths."""
    lt = np.asarray(log_trans, np.float64)
    st = np.asarray(state_types)
    lM, lI, lD = _log_tkf_tables(sub_matrix, pi)
    ll, paths = _lib.sample_paths(st, np.zeros(st.size, np.int32), 1, xs, ys, lt[None], lM, lI, lD,
                                  int(n_samples), _seed_of(seed), device=_device())
    return ll, [[[tuple(int(v) for v in row) for row in pth] for pth in per_pair] for per_pair in paths]


def sample_traceback_2d(log_trans, state_types, x_seq, y_seq, sub_matrix, pi, rng_key):
    """sample_traceback_2d (dp/hmm.py:2043-2101): (log_prob, one path sampled
    from the posterior as a list of (i, j, state)).  rng_key: an int or an
    integer array (a PRNG key) seeding the device stream."""
    ll, paths = sample_traceback_2d_batch(log_trans, state_types, [np.asarray(x_seq)], [np.asarray(y_seq)],
                                          sub_matrix, pi, 1, rng_key)
    return float(ll[0]), paths[0][0]


def exact_suffstats_batch(n_chi_stack, main_ins, main_del, t_array, dom_ins, dom_del, dom_weights,
                          frag_weights, ext_rates):
    """Exact MixDom2 sufficient statistics from collapsed counts
    (models/exact_suffstats_batch.py:485-541); see pairhmm.suffstats."""
    from . import suffstats
    return suffstats.exact_suffstats_batch(n_chi_stack, main_ins, main_del, t_array, dom_ins, dom_del,
                                           dom_weights, frag_weights, ext_rates)


def estep_batch_mixdom2(params, xs, ys, ts, with_class_counts=True, exact_suffstats=False):
    """Batched MixDom2 E-step over pairs of any lengths in one persistent
    launch (replaces the bucketed jit(vmap(forward_backward_2d)) callers).

    Returns a dict of device tensors: log_p [P], n_trans [P,N,N], cnt_M
    [P,G,21,21], cnt_I/cnt_D [P,G,21], status [P]; with with_class_counts,
    the per-pair class counts of e_step_mixdom2 and their Holmes-Rubin
    statistics class_W [P,C,A], class_U [P,C,A,A]; with exact_suffstats, under
    'suffstats', the per-pair exact sufficient statistics of the exploded
    model (exact_suffstats_batch on n_trans)."""
    dev = _device()
    pro = _lib.MixDom2Prologue(params)
    K, F = pro.K, pro.F
    plan = get_plan(pm.mixdom_state_types(K, F), pm.mixdom_state_groups(K, F), K * F)
    if with_class_counts and not exact_suffstats:
        # a batch shape seen before replays its captured CUDA graph (pairhmm.graphs)
        g = graphs.mixdom2_estep(pro, xs, ys, ts, dev, tuned_plan=plan)
        if g is not None:
            res = {'log_p': g['ll']}
            res.update({k: v for k, v in g.items() if k != 'll'})
            return res
    t_dev = (ts if isinstance(ts, torch.Tensor) else torch.from_numpy(
        np.ascontiguousarray(np.asarray(ts, np.float64).reshape(-1)))).to(device=dev, dtype=torch.float64)
    if pro.nest_supported():   # the kernels contract this layout through the factored record
        chi, EM, EI, ED, csubs, nest = pro(t_dev, device=dev, with_nest=True)
    else:
        (chi, EM, EI, ED, csubs), nest = pro(t_dev, device=dev), None
    b = _lib.make_batch(xs, ys, chi, EM, EI, ED, device=dev, nest=nest, nest_kf=(K, F))
    autotune.apply_cached(plan, b)
    # every output in one device buffer: one copy brings them all to the host
    P, N, G, C, A = b.n_pairs, 2 + 5 * K * F, K * F, pro.C, pro.A
    f64 = torch.float64
    specs = [('ll', (P,), f64), ('n_trans', (P, N, N), f64), ('cnt_M', (P, G, 21, 21), f64),
             ('cnt_I', (P, G, 21), f64), ('cnt_D', (P, G, 21), f64), ('status', (P,), torch.int32)]
    use_arena = with_class_counts and C <= 8
    if use_arena:
        specs += [(k, sh, f64) for k, sh in pro.class_count_shapes(P).items()]
        specs += [('class_W', (P, C, A), f64), ('class_U', (P, C, A, A), f64)]
    ar = _lib.OutputArena(dev, specs)
    out = _lib.estep(plan, b, out={k: ar[k] for k in ('ll', 'n_trans', 'cnt_M', 'cnt_I', 'cnt_D', 'status')})
    res = {'log_p': out['ll'], 'n_trans': out['n_trans'], 'cnt_M': out['cnt_M'],
           'cnt_I': out['cnt_I'], 'cnt_D': out['cnt_D'], 'status': out['status']}
    if with_class_counts:
        if use_arena:
            res.update(pro.class_counts(csubs, out['cnt_M'], out['cnt_I'], out['cnt_D'],
                                        out={k: ar[k] for k in pro.class_count_shapes(P)}))
            W, U = holmes_rubin_batch(params['class_S_exch'], params['class_pis'], t_dev,
                                      res['class_match_counts'], out=(ar['class_W'], ar['class_U']))
        else:
            res.update(class_split(params, out['cnt_M'], out['cnt_I'], out['cnt_D'], csubs=csubs))
            W, U = holmes_rubin_batch(params['class_S_exch'], params['class_pis'], t_dev,
                                      res['class_match_counts'])
        res['class_W'], res['class_U'] = W, U
    if exact_suffstats:
        res['suffstats'] = exact_suffstats_batch(out['n_trans'], params['main_ins'], params['main_del'], ts,
                                                 params['dom_ins'], params['dom_del'], params['dom_weights'],
                                                 params['frag_weights'], params['ext_rates'])
    return res


def e_step_mixdom2(params, x, y):
    """MixDom2 E-step (train/likelihood.py:143-373): (LL, n_trans, dict with
    class_W, class_U, class_match_counts, class_insert_counts,
    class_delete_counts, classdist_counts)."""
    r = estep_batch_mixdom2(params, [np.asarray(x)], [np.asarray(y)], np.array([params['t']]))
    keys = ('class_W', 'class_U', 'class_match_counts', 'class_insert_counts', 'class_delete_counts',
            'classdist_counts')
    host = to_host({k: r[k] for k in keys + ('log_p', 'n_trans')})
    out = {k: host[k][0] for k in keys}
    return float(host['log_p'][0]), host['n_trans'][0], out


# ---------------------------------------------------------------- differentiable log-likelihood
class PairHMMLogLik(torch.autograd.Function):
    """Sum of per-pair log-likelihoods with the score-identity adjoint.

    forward runs the CUDA E-step; backward returns
      dLL/dchi[s,k]   = n_trans[s,k] / chi[s,k]
      dLL/dEM[g,a,b]  = cnt_M[g,a,b] / EM[g,a,b]   (and I, D alike)
    so torch autograd through the float64 builders of chi(theta) and the
    emission tables delivers dLL/dtheta for every parameter -- the score
    identity the reference's custom VJPs implement (train/vjp.py:130-329,
    388-458, 682-818)."""

    @staticmethod
    def forward(ctx, chi, EM, EI, ED, plan, xs, ys):
        dev = chi.device
        b = _lib.make_batch(xs, ys, chi.detach(), EM.detach(), EI.detach(), ED.detach(), device=dev)
        out = _lib.estep(plan, b)
        ctx.save_for_backward(chi, EM, EI, ED, out['n_trans'], out['cnt_M'], out['cnt_I'], out['cnt_D'])
        ctx.per_pair = (chi.shape[0] == len(xs), EM.shape[0] == len(xs))
        ctx.status = out['status']
        return out['ll']

    @staticmethod
    def backward(ctx, g):
        chi, EM, EI, ED, n, cM, cI, cD = ctx.saved_tensors
        gw = g.to(torch.float64)

        def ratio(cnt, tab, per_pair):
            r = torch.where(tab > 0, cnt / torch.where(tab > 0, tab, torch.ones_like(tab)),
                            torch.zeros_like(cnt))
            shape = (-1,) + (1,) * (cnt.dim() - 1)
            r = r * gw.reshape(shape)
            return r if per_pair else r.sum(dim=0, keepdim=True)
        pc, pe = ctx.per_pair
        return (ratio(n, chi, pc).to(chi.dtype), ratio(cM, EM, pe).to(EM.dtype),
                ratio(cI, EI, pe).to(EI.dtype), ratio(cD, ED, pe).to(ED.dtype), None, None, None)


class MixDom2Chi(torch.autograd.Function):
    """The collapsed MixDom chi [P,N,N] (float64) built on the device
    (phmm_mixdom2_chi), differentiable in main_ins, main_del, t, dom_ins,
    dom_del, dom_weights, frag_weights and ext_rates: the backward pass is the
    device vector-Jacobian product phmm_mixdom2_chi_vjp (forward-mode dual
    numbers through the same builder), replacing autograd through the float64
    torch builder of models/mixdom.py:104-423."""

    @staticmethod
    def forward(ctx, pro, t, main_ins, main_del, dom_ins, dom_del, dom_w, frag_w, ext):
        tt = t.detach().to(torch.float64).reshape(-1).contiguous()
        _, chi64 = pro.chi(tt)
        ctx.pro = pro
        ctx.ext_diag = ext.dim() == 2
        ctx.shapes = [v.shape for v in (t, main_ins, main_del, dom_ins, dom_del, dom_w, frag_w, ext)]
        ctx.save_for_backward(tt)
        return chi64

    @staticmethod
    def backward(ctx, g):
        tt, = ctx.saved_tensors
        pro = ctx.pro
        K, F = pro.K, pro.F
        gr = pro.chi_vjp(tt, g)
        sh = ctx.shapes
        out = [gr[:, 2].reshape(sh[0]) if tt.numel() == int(np.prod(sh[0])) else gr[:, 2].sum().reshape(sh[0]),
               gr[:, 0].sum().reshape(sh[1]), gr[:, 1].sum().reshape(sh[2])]
        j = 3
        for n, shape in ((K, sh[3]), (K, sh[4]), (K, sh[5]), (K * F, sh[6])):
            out.append(gr[:, j:j + n].sum(0).reshape(shape))
            j += n
        gext = gr[:, j:j + K * F * F].sum(0).reshape(K, F, F)
        out.append(torch.diagonal(gext, dim1=-2, dim2=-1).reshape(sh[7]) if ctx.ext_diag else gext.reshape(sh[7]))
        return (None, *out)


def mixdom2_log_prob(main_ins_rate, main_del_rate, t, dom_ins_rates, dom_del_rates, dom_weights,
                     frag_weights, ext_rates, class_pis, class_S_exch, class_dist, x_seq, y_seq):
    """log P(x, y) under MixDom2 with gradients for every tensor argument
    (train/vjp.py:627-680).  Arguments may be float64 torch tensors with
    requires_grad; x_seq/y_seq may also be lists of sequences, in which case
    t is a [P] tensor of per-pair times and the result is [P]."""
    dev = _device()
    batched = isinstance(x_seq, (list, tuple))
    xs = list(x_seq) if batched else [np.asarray(x_seq)]
    ys = list(y_seq) if batched else [np.asarray(y_seq)]
    tt = pm._t(t, device=dev).reshape(-1)
    f = lambda v: pm._t(v, device=dev)
    K, F = f(frag_weights).shape
    if K * F <= 33 and f(class_pis).shape[-1] == 20:
        # chi and its gradient on the device (phmm_mixdom2_chi / _chi_vjp)
        pro = _lib.MixDom2Prologue({
            'main_ins': main_ins_rate, 'main_del': main_del_rate, 'dom_ins': dom_ins_rates,
            'dom_del': dom_del_rates, 'dom_weights': dom_weights, 'frag_weights': frag_weights,
            'ext_rates': ext_rates, 'class_pis': class_pis, 'class_S_exch': class_S_exch,
            'classdist': class_dist})
        chi = MixDom2Chi.apply(pro, tt, f(main_ins_rate), f(main_del_rate), f(dom_ins_rates), f(dom_del_rates),
                               f(dom_weights), f(frag_weights), f(ext_rates))
    else:
        chi = pm.build_nested_trans(f(main_ins_rate), f(main_del_rate), tt, f(dom_ins_rates),
                                    f(dom_del_rates), f(dom_weights), f(frag_weights), f(ext_rates))
    csubs = pm.class_subs(f(class_S_exch), f(class_pis), tt)
    EM, EI, ED = pm.tables_per_class(csubs, f(class_pis), f(class_dist))
    plan = get_plan(pm.mixdom_state_types(K, F), pm.mixdom_state_groups(K, F), K * F)
    ll = PairHMMLogLik.apply(chi, EM, EI, ED, plan, xs, ys)
    return ll if batched else ll[0]


def mixdom_log_prob(main_ins_rate, main_del_rate, t, dom_ins_rates, dom_del_rates, dom_weights,
                    frag_weights, ext_rates, Q, pi, x_seq, y_seq):
    """log P(x, y) under the nested MixDom pair HMM with one substitution
    model (train/vjp.py:351-458): chi from build_nested_trans, every M/I/D
    state emitting through pair_hmm_emissions(P(t), pi).  Gradients for every
    tensor argument through the score identity, as mixdom2_log_prob."""
    dev = _device()
    batched = isinstance(x_seq, (list, tuple))
    xs = list(x_seq) if batched else [np.asarray(x_seq)]
    ys = list(y_seq) if batched else [np.asarray(y_seq)]
    tt = pm._t(t, device=dev).reshape(-1)
    f = lambda v: pm._t(v, device=dev)
    K, F = f(frag_weights).shape
    chi = pm.build_nested_trans(f(main_ins_rate), f(main_del_rate), tt, f(dom_ins_rates),
                                f(dom_del_rates), f(dom_weights), f(frag_weights), f(ext_rates))
    sub = pm.transition_matrix(f(Q), tt)
    EM, EI, ED = pm.tables_tkf(sub, f(pi))
    st = pm.mixdom_state_types(K, F)
    plan = get_plan(st, np.zeros(len(st), np.int32), 1)
    ll = PairHMMLogLik.apply(chi, EM, EI, ED, plan, xs, ys)
    return ll if batched else ll[0]


def _tkf_log_prob(model, ins_rate, del_rate, t, ext, Q, pi, x_seq, y_seq):
    dev = _device()
    f = lambda v: pm._t(v, device=dev)
    tt = f(t).reshape(-1)
    if model == 'tkf91':
        chi = pm.tkf91_trans(f(ins_rate), f(del_rate), tt)
    elif model == 'tkf91_cond':
        chi = pm.tkf91_trans_cond(f(ins_rate), f(del_rate), tt)
    else:
        chi = pm.tkf92_trans(f(ins_rate), f(del_rate), tt, f(ext))
    sub = pm.transition_matrix(f(Q), tt)
    EM, EI, ED = pm.tables_tkf(sub, f(pi))
    plan = get_plan(np.array([S, M, I, D, E]), np.zeros(5, np.int32), 1)
    return PairHMMLogLik.apply(chi, EM, EI, ED, plan, [np.asarray(x_seq)], [np.asarray(y_seq)])[0]


def tkf91_log_prob(ins_rate, del_rate, t, Q, pi, x_seq, y_seq):
    """log P(x,y) under TKF91, differentiable in all float arguments (train/vjp.py:109-194)."""
    return _tkf_log_prob('tkf91', ins_rate, del_rate, t, None, Q, pi, x_seq, y_seq)


def tkf91_log_prob_cond(ins_rate, del_rate, t, Q, pi, x_seq, y_seq):
    """log P(x,y | ancestor length) + const under TKF91 (train/vjp.py:198-249),
    differentiable in all float arguments."""
    return _tkf_log_prob('tkf91_cond', ins_rate, del_rate, t, None, Q, pi, x_seq, y_seq)


def tkf92_log_prob(ins_rate, del_rate, t, ext, Q, pi, x_seq, y_seq):
    """log P(x,y) under TKF92, differentiable in all float arguments (train/vjp.py:252-329)."""
    return _tkf_log_prob('tkf92', ins_rate, del_rate, t, ext, Q, pi, x_seq, y_seq)


def observed_ll(model, params, x, y):
    """log P(x, y | theta), differentiable (train/likelihood.py:415-460)."""
    if model == 'tkf91':
        return tkf91_log_prob(params['ins_rate'], params['del_rate'], params['t'], params['Q'],
                              params['pi'], x, y)
    if model == 'tkf92':
        return tkf92_log_prob(params['ins_rate'], params['del_rate'], params['t'], params['ext'],
                              params['Q'], params['pi'], x, y)
    if model == 'mixdom2':
        return mixdom2_log_prob(params['main_ins'], params['main_del'], params['t'], params['dom_ins'],
                                params['dom_del'], params['dom_weights'], params['frag_weights'],
                                params['ext_rates'], params['class_pis'], params['class_S_exch'],
                                params['classdist'], x, y)
    raise ValueError(f'Unknown model: {model}')


# ---------------------------------------------------------------- batched TKF92 (train/tkf92_svi_bw.py)
def _tkf92_batch(xs_pad, ys_pad, ts, Lx_real, Ly_real, lam, mu, ext, Q, pi):
    dev = _device()
    # chi floored at 1e-30 (log(max(tau, 1e-30)), tkf92_svi_bw.py:164), P(t) and
    # the emission tables: the device prologue phmm_tkf92_tables
    chi, EM, EI, ED, _ = _lib.tkf92_tables(lam, mu, ext, Q, pi, ts, device=dev)
    Lx_real = np.asarray(Lx_real).reshape(-1)
    Ly_real = np.asarray(Ly_real).reshape(-1)
    xs = [np.asarray(xs_pad[b])[:int(Lx_real[b])] for b in range(len(Lx_real))]
    ys = [np.asarray(ys_pad[b])[:int(Ly_real[b])] for b in range(len(Ly_real))]
    plan = get_plan(np.array([S, M, I, D, E]), np.zeros(5, np.int32), 1)
    return plan, _lib.make_batch(xs, ys, chi, EM, EI, ED, device=dev)


def estep_batch_tkf92_forward_only(xs_pad, ys_pad, ts, Lx_real, Ly_real, lam, mu, ext, Q, pi):
    """Per-pair log_p of pre-padded pairs (train/tkf92_svi_bw.py:337-365)."""
    plan, b = _tkf92_batch(xs_pad, ys_pad, ts, Lx_real, Ly_real, lam, mu, ext, Q, pi)
    ll, st = _lib.forward(plan, b)
    return ll


def estep_batch_tkf92(xs_pad, ys_pad, ts, Lx_real, Ly_real, lam, mu, ext, Q, pi):
    """Batched TKF92 E-step (train/tkf92_svi_bw.py:263-334): dict of device
    tensors 'log_p', 'B', 'D', 'S' (BDI statistics), 'L', 'M' (kappa
    coefficients), 'T', 'ext_count', 'notext_count', 'n_chi_diag' [P,5,5]
    and 'status'.  The DP runs on the GPU; the chi decomposition and the BDI
    statistics are the float64 epilogue of pairhmm.bdi."""
    from . import bdi
    plan, b = _tkf92_batch(xs_pad, ys_pad, ts, Lx_real, Ly_real, lam, mu, ext, Q, pi)
    out = _lib.estep(plan, b)
    res = bdi.tkf92_bdi_epilogue(out['n_trans'], lam, mu, np.asarray(ts, np.float64), ext)
    res.pop('n_trans_resolved')
    res.update({'log_p': out['ll'], 'n_chi_diag': out['n_trans'], 'status': out['status']})
    return res


def _mixfrag_batch(xs_pad, ys_pad, ts, Lx_real, Ly_real, lam, mu, exts, weights, Q, pi):
    dev = _device()
    F = int(np.asarray(exts).size)
    tt = torch.as_tensor(np.asarray(ts, np.float64).reshape(-1))
    # chi floored at 1e-30 as the reference takes log(max(tau, 1e-30)) (mixfrag_svi_bw.py:136)
    chi = torch.clamp(pm.mixfrag_trans_batch(lam, mu, tt, exts, weights), min=1e-30)
    EM, EI, ED = pm.tables_tkf(pm.transition_matrix(pm._t(Q), tt), pm._t(pi))
    Lx_real = np.asarray(Lx_real).reshape(-1)
    Ly_real = np.asarray(Ly_real).reshape(-1)
    xs = [np.asarray(xs_pad[b])[:int(Lx_real[b])] for b in range(len(Lx_real))]
    ys = [np.asarray(ys_pad[b])[:int(Ly_real[b])] for b in range(len(Ly_real))]
    st = pm.mixfrag_state_types(F)
    plan = get_plan(st, np.zeros(st.size, np.int32), 1)
    return plan, _lib.make_batch(xs, ys, chi, EM, EI, ED, device=dev)


def estep_batch_mixfrag_forward_only(xs_pad, ys_pad, ts, Lx_real, Ly_real, lam, mu, exts, weights, Q, pi):
    """Per-pair log_p of pre-padded pairs under MixFrag (TKF92 with F fragment
    types; train/mixfrag_svi_bw.py:236-250)."""
    plan, b = _mixfrag_batch(xs_pad, ys_pad, ts, Lx_real, Ly_real, lam, mu, exts, weights, Q, pi)
    ll, st = _lib.forward(plan, b)
    return ll


def estep_batch_mixfrag(xs_pad, ys_pad, ts, Lx_real, Ly_real, lam, mu, exts, weights, Q, pi):
    """Batched MixFrag E-step (train/mixfrag_svi_bw.py:194-232): dict of device
    tensors 'log_p', 'B', 'D', 'S' (BDI statistics of the fragment-resolved
    counts), 'L', 'M' (kappa coefficients), 'T', 'F_f' / 'E_f' [P, F]
    (fragment-extension and fragment-end counts per fragment type), plus
    'n_chi' [P, 3F+2, 3F+2] and 'status'.  The DP runs on the GPU; the
    resolution and the BDI statistics are the float64 epilogue of pairhmm.bdi."""
    from . import bdi
    plan, b = _mixfrag_batch(xs_pad, ys_pad, ts, Lx_real, Ly_real, lam, mu, exts, weights, Q, pi)
    out = _lib.estep(plan, b)
    res = bdi.mixfrag_bdi_epilogue(out['n_trans'], lam, mu, np.asarray(ts, np.float64), exts, weights)
    res.update({'log_p': out['ll'], 'n_chi': out['n_trans'], 'status': out['status']})
    return res


def tkf92_log_prob_fb(lam, mu, ext, t, Q, pi, x_seq, y_seq, real_Lx=None, real_Ly=None):
    """log P(x, y | TKF92(lam, mu, ext), Q, pi, t) (train/tkf92_adam_fb.py:77-104):
    the TKF92 matrix floored at 1e-30 in log space, differentiable in every
    float argument (score identity over the CUDA E-step).  With real_Lx /
    real_Ly the sequences are taken as padded and cut to those lengths."""
    dev = _device()
    f = lambda v: pm._t(v, device=dev)
    x = np.asarray(x_seq)
    y = np.asarray(y_seq)
    if real_Lx is not None:
        x = x[:int(real_Lx)]
    if real_Ly is not None:
        y = y[:int(real_Ly)]
    tt = f(t).reshape(-1)
    chi = torch.clamp(pm.tkf92_trans(f(lam), f(mu), tt, f(ext)), min=1e-30)
    EM, EI, ED = pm.tables_tkf(pm.transition_matrix(f(Q), tt), f(pi))
    plan = get_plan(np.array([S, M, I, D, E]), np.zeros(5, np.int32), 1)
    return PairHMMLogLik.apply(chi, EM, EI, ED, plan, [x], [y])[0]
