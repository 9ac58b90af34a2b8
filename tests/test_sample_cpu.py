"""The oracle of the stochastic forward traceback (oracle/sample.py): its
draws follow the posterior over alignments (frequencies against the exact
path probabilities of a small lattice, enumerated), and every path is a
valid alignment path."""
import numpy as np


def enumerate_paths(lt, st, emit, Lx, Ly):
    """{path tuple: probability} over all state paths from (0,0,S) to (Lx,Ly)."""
    from oracle.models import M, I, D
    e_idx = int(np.argmax(st == 4))
    out = {}

    def rec(i, j, k, path, logp):
        if i == Lx and j == Ly and k != 0:
            out[tuple(path)] = logp + lt[k, e_idx]
        for k2 in range(st.size):
            t = st[k2]
            if t == M and i < Lx and j < Ly:
                ni, nj = i + 1, j + 1
            elif t == I and j < Ly:
                ni, nj = i, j + 1
            elif t == D and i < Lx:
                ni, nj = i + 1, j
            else:
                continue
            rec(ni, nj, k2, path + [(ni, nj, k2)], logp + lt[k, k2] + emit[ni, nj, k2])
    rec(0, 0, 0, [(0, 0, 0)], 0.0)
    keys = list(out)
    lp = np.array([out[k] for k in keys])
    pr = np.exp(lp - lp.max())
    return dict(zip(keys, pr / pr.sum())), float(np.log(np.exp(lp - lp.max()).sum()) + lp.max())


def small_case(seed=3):
    from oracle import dp, models as om
    rng = np.random.default_rng(seed)
    A = 20
    pi = rng.dirichlet(np.ones(A))
    Sx = rng.lognormal(0, 1, (A, A))
    Sx = np.triu(Sx, 1) + np.triu(Sx, 1).T
    Q = Sx * pi[None, :]
    np.fill_diagonal(Q, -Q.sum(axis=1))
    t = 0.7
    lt = om.safe_log(om.tkf91_trans(0.3, 0.35, t))
    st = np.array([0, 1, 2, 3, 4])
    sub = om.transition_matrix(Q, t)
    EM, EI, ED = dp.group_tables_tkf(sub, pi)
    x, y = rng.integers(0, 20, 2), rng.integers(0, 20, 3)
    emit = dp.log_emission_table(st, np.zeros(5, int), x, y, EM, EI, ED)
    return lt, st, emit, x, y, sub, pi


def test_oracle_sampler_follows_posterior():
    from oracle import sample
    lt, st, emit, x, y, _, _ = small_case()
    exact, ll_enum = enumerate_paths(lt, st, emit, len(x), len(y))
    ll, paths = sample.sample_paths(lt, st, emit, 6000, seed=11)
    assert abs(ll - ll_enum) < 1e-10
    freq = {}
    for pth in paths:
        freq[tuple(pth)] = freq.get(tuple(pth), 0) + 1
    assert set(freq) <= set(exact)
    n = len(paths)
    for k, p in exact.items():
        # 5 standard deviations of a binomial proportion
        assert abs(freq.get(k, 0) / n - p) <= 5 * np.sqrt(p * (1 - p) / n) + 1e-9, (k, p)


def test_oracle_stream_is_deterministic():
    from oracle import sample
    lt, st, emit, _, _, _, _ = small_case(5)
    _, a = sample.sample_paths(lt, st, emit, 20, seed=7)
    _, b = sample.sample_paths(lt, st, emit, 20, seed=7)
    _, c = sample.sample_paths(lt, st, emit, 20, seed=8)
    assert a == b and a != c
