"""The factored MixDom transitions (pairhmm.models.nested_record, the input
of the two-warp stripes' factored contraction) against the oracle's dense chi
(oracle/models.py build_nested_trans, pinned to the reference's
models/mixdom.py:252-423): chi[2+s, 2+k] = exit[s] cin[U(s)][k] + [d_s = d_k]
intra[d][s', k'] for every body pair, to float64 rounding."""
import numpy as np
import pytest
import torch

from oracle import models as om
from pairhmm import models as pm, synth


@pytest.mark.parametrize('K,F,C', [(1, 1, 1), (3, 1, 1), (2, 2, 2), (4, 2, 2), (8, 4, 4), (2, 3, 1)])
@pytest.mark.parametrize('mixdom1_ext', [False, True])
def test_record_rebuilds_oracle_chi(K, F, C, mixdom1_ext):
    rng = np.random.default_rng(11 * K + F)
    p = synth.mixdom2_params(rng, K, F, C)
    ext = np.asarray(p['ext_rates'], np.float64)
    if mixdom1_ext and ext.ndim == 3:   # (K, F) per-fragment extension (MixDom1 form)
        ext = np.stack([np.diag(e) for e in ext])
    ts = np.array([0.05, 0.6, 2.0])
    rec = pm.nested_record(p['main_ins'], p['main_del'], torch.as_tensor(ts), p['dom_ins'], p['dom_del'],
                           p['dom_weights'], p['frag_weights'], ext).numpy()
    assert rec.shape == (3, pm.nest_record_len(K, F))
    nb, bs = 5 * K * F, 5 * F
    U = np.tile(np.repeat([0, 0, 0, 1, 2], F), K)
    for i, t in enumerate(ts):
        chi = om.build_nested_trans(p['main_ins'], p['main_del'], t, p['dom_ins'], p['dom_del'],
                                    p['dom_weights'], p['frag_weights'], ext)
        exit_, cin = rec[i, :nb], rec[i, nb:4 * nb].reshape(3, nb)
        intra = rec[i, 4 * nb:].reshape(K, bs, bs)
        body = exit_[:, None] * cin[U, :]
        for d in range(K):
            body[d * bs:(d + 1) * bs, d * bs:(d + 1) * bs] += intra[d]
        np.testing.assert_allclose(body, chi[2:, 2:], rtol=1e-12, atol=1e-15)
        # the structural zeros of the same-domain blocks: MM/MI/MD couple
        # only among themselves, II and DD only within their own sub-state
        sub = np.repeat(np.array([0, 0, 0, 1, 2]), F)
        assert np.all(intra[:, sub[:, None] != sub[None, :]] == 0.0)
        assert np.all(rec[i] >= 0.0)


def test_library_reports_the_factored_layouts():
    """phmm_nest_supported (a host query, no GPU): the 17-state two-warp layout
    and the wide kernels' F = 4 layouts with 4..8 domains."""
    from pairhmm import _lib
    lib = _lib.load()
    assert lib.phmm_nest_supported(3, 1) == 1
    for K in range(4, 9):
        assert lib.phmm_nest_supported(K, 4) == 1
    for K, F in [(1, 1), (2, 1), (4, 1), (2, 2), (4, 2), (3, 4), (9, 4), (8, 2)]:
        assert lib.phmm_nest_supported(K, F) == 0, (K, F)
