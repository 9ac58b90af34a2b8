"""FP64 oracle: masked 2D forward-backward variants (TEST INFRASTRUCTURE ONLY).

Part of the CPU oracle the test-suite checks the product's cell-masked
E-step against; the product never imports it.

Restates in NumPy float64, on top of ``oracle.dp.forward_backward``:
  * ``mask_emissions_match_aligned`` (dp/hmm.py:1085-1117): M-type emissions
    are NEG_INF except at grid cells (mi+1, mj+1) of the training alignment;
  * ``forward_backward_2d_banded`` (dp/hmm.py:2104-2492): the forward and
    backward recursions restricted to the cells with |j - c_i| <= W around
    the band centres c_i, W = pad_to_bin(band_width) (dp/hmm.py:66-98).  A
    banded recursion equals the full one with every emission outside the
    band set to NEG_INF (no path leaves the band); posteriors are returned
    in the reference's band layout (pad_to_bin(Lx)+1, 2W+1, N), position
    (i, b) holding column j = c_i - W + b, rows past Lx centred on Ly.

Pinned against ``tests/golden/masked.npz`` (the reference's own outputs,
``tests/golden/make_golden_masked.py``).  For Lx that is not a padding bin
the reference's banded backward starts from the terminal band placed at
row pad_to_bin(Lx) (dp/hmm.py:2337-2343) and its posteriors and counts are
not those of the banded model (its expected transitions sum to about 1 for
a path of 20+ steps); this oracle follows the banded model, which is the
reference's result whenever Lx is a bin size.
"""
from __future__ import annotations

import numpy as np

from .dp import forward_backward
from .models import M, NEG_INF

BIN_BASE, BIN_MAX, BIN_MULT = 4, 4096, 1.2


def _bins():
    out = [BIN_BASE]
    v = float(BIN_BASE)
    while v < BIN_MAX:
        v *= BIN_MULT
        b = int(round(v))
        if b > out[-1]:
            out.append(b)
    if out[-1] < BIN_MAX:
        out.append(BIN_MAX)
    return [0, 1, 2, 3] + out


def pad_to_bin(n):
    """dp/hmm.py:66-98 without the environment cap."""
    n = max(int(n), 1)
    for b in _bins():
        if b >= n:
            return b
    return int(2 ** np.ceil(np.log2(n)))


def mask_emissions_match_aligned(emit, state_types, match_i, match_j):
    """emit (Lx+1, Ly+1, N) with M-state entries NEG_INF off the alignment's
    match cells (mi+1, mj+1) (dp/hmm.py:1085-1117)."""
    emit = np.array(emit, dtype=float)
    allowed = np.zeros(emit.shape[:2], bool)
    allowed[np.asarray(match_i, int) + 1, np.asarray(match_j, int) + 1] = True
    isM = np.asarray(state_types) == M
    emit[:, :, isM] = np.where(allowed[:, :, None], emit[:, :, isM], emit[:, :, isM] + NEG_INF)
    return emit


def band_allowed(Lx, Ly, band_center, W):
    """(Lx+1, Ly+1) bool: |j - c_i| <= W."""
    c = np.asarray(band_center, int)[:Lx + 1]
    j = np.arange(Ly + 1)
    return np.abs(j[None, :] - c[:, None]) <= W


def forward_backward_banded(log_trans, state_types, emit, band_center, band_width):
    """(log_prob, posteriors in band layout, expected_trans) of
    forward_backward_2d_banded for a full emission table emit (Lx+1, Ly+1, N)."""
    emit = np.array(emit, dtype=float)
    Lx, Ly = emit.shape[0] - 1, emit.shape[1] - 1
    W = pad_to_bin(band_width)
    ok = band_allowed(Lx, Ly, band_center, W)
    emit[~ok] = NEG_INF
    if not ok[0, 0]:
        N = emit.shape[2]
        ll, post, n = NEG_INF, np.zeros_like(emit), np.zeros((N, N))
    else:
        ll, post, n, _, _ = forward_backward(log_trans, state_types, emit)
    return ll, to_band_layout(post, band_center, W), n


def to_band_layout(dense, band_center, W):
    """(Lx+1, Ly+1, N) -> (pad_to_bin(Lx)+1, 2W+1, N), zero off the lattice."""
    Lx, Ly, N = dense.shape[0] - 1, dense.shape[1] - 1, dense.shape[2]
    Lp = pad_to_bin(Lx)
    out = np.zeros((Lp + 1, 2 * W + 1, N))
    c = np.full(Lp + 1, Ly)
    c[:Lx + 1] = np.asarray(band_center, int)[:Lx + 1]
    for i in range(Lx + 1):
        for b in range(2 * W + 1):
            j = c[i] - W + b
            if 0 <= j <= Ly:
                out[i, b] = dense[i, j]
    return out
