"""The X/A/Y pair-record reader and helpers (pairhmm.pair_format, the native
phmm_pairs_count / phmm_pairs_decode) against the reference's own
util/pair_format.py outputs (tests/golden/pairs.jsonl, pairs.npz)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden


@pytest.fixture(scope='module')
def lib():
    from pairhmm import build, _lib
    build.build()
    return _lib.load()


def _text():
    with open(os.path.join(GOLDEN, 'pairs.jsonl')) as f:
        return f.read()


def test_native_reader_matches_reference_decode(lib):
    from pairhmm import pair_format as pf
    g = load_golden('pairs')
    r = pf.read_records(_text())
    assert r.n_pairs == int(g['n_pairs'])
    for p in range(r.n_pairs):
        pre = f'p{p}_'
        x, y, st, anc, desc, t = r.decoded(p)
        assert np.array_equal(x, g[pre + 'x_int']) and np.array_equal(y, g[pre + 'y_int'])
        assert st == list(g[pre + 'states'])
        assert anc == list(g[pre + 'anc_chars']) and desc == list(g[pre + 'desc_chars'])
        assert t == float(g[pre + 't_est'])
        assert r.fam[p] == str(g[pre + 'fam'])
        # the batch layout: pair p as [x_p, y_p]
        assert r.y_off[p] == r.x_off[p] + r.Lx[p]
        mi, mj = r.match_positions(p)
        m = np.asarray(st) == 1
        assert np.array_equal(r.x(p)[mi], np.asarray(r.columns(p)[1])[m])
        assert np.array_equal(r.y(p)[mj], np.asarray(r.columns(p)[2])[m])


def test_python_helpers_match_reference():
    from pairhmm import pair_format as pf
    g = load_golden('pairs')
    lines = _text().strip().split('\n')
    for p, line in enumerate(lines):
        pre = f'p{p}_'
        ref = json.loads(line)
        kw = {k: ref[k] for k in ('gamma',) if k in ref}
        mine = pf.encode_pair(g[pre + 'anc_in'], g[pre + 'desc_in'], list(g[pre + 'states_in']),
                              float(g[pre + 't_in']), str(g[pre + 'fam']), f'r{p}a', f'r{p}b',
                              gamma_labels=kw.get('gamma'), gamma_log_posteriors=ref.get('gamma_lp'))
        assert mine == ref
        x, y, st, anc, desc, t, gl, glp = pf.decode_pair(ref)
        assert st == list(g[pre + 'states']) and anc == list(g[pre + 'anc_chars'])
        assert pf.rle_encode(pf.rle_decode(ref['a'])) == ref['a']
    for k in range(4):
        rec = json.loads(str(g[f'bad{k}_record']))
        assert pf.validate_record(rec) == (bool(g[f'bad{k}_ok']), str(g[f'bad{k}_msg']))


@pytest.mark.parametrize('bad,msg', [
    ('{"x": "ACD", "a": "M2", "y": "AC", "t": 0.1}', 'M+D=2 != len(X)=3'),
    ('{"x": "AC", "a": "M2I1", "y": "AC", "t": 0.1}', 'M+I=3 != len(Y)=2'),
    ('{"x": "ABC", "a": "M3", "y": "ACD", "t": 0.1}', "invalid residue 'B' in X"),
    ('{"x": "AC", "a": "M2", "y": "AC"}', 'needs keys'),
    ('{"x": "AC", "a": "M2", "y": "AC", "t": 0.1', "expected ','"),
])
def test_native_reader_errors_name_the_line(lib, bad, msg):
    from pairhmm import pair_format as pf, _lib
    good = _text().split('\n')[0]
    with pytest.raises(_lib.PairHMMError) as e:
        pf.read_records(good + '\n\n' + bad + '\n')
    assert 'line 3' in str(e.value) and msg in str(e.value)


def test_empty_and_blank_text(lib):
    from pairhmm import pair_format as pf
    assert pf.read_records('').n_pairs == 0
    assert pf.read_records('\n  \n').n_pairs == 0


def test_native_reader_survives_mutated_records(lib):
    """Truncated, mutated and random lines either parse to the same answer as
    the Python decoder or raise PairHMMError; the reader never crashes."""
    from pairhmm import pair_format as pf, _lib
    rng = np.random.default_rng(2026)
    lines = _text().strip().split('\n')
    alphabet = list('{}[]":,. xaytfm0123456789MIDACDEFGHIKLMNPQRSTVWYBZ\\\t')
    for trial in range(400):
        line = lines[int(rng.integers(len(lines)))]
        kind = trial % 4
        if kind == 0:
            line = line[:int(rng.integers(len(line) + 1))]
        elif kind == 1:
            pos = int(rng.integers(len(line)))
            line = line[:pos] + alphabet[int(rng.integers(len(alphabet)))] + line[pos + 1:]
        elif kind == 2:
            pos = int(rng.integers(len(line)))
            line = line[:pos] + line[pos + 1:]
        else:
            line = ''.join(alphabet[int(v)] for v in rng.integers(0, len(alphabet), int(rng.integers(1, 80))))
        try:
            r = pf.read_records(line + '\n')
        except _lib.PairHMMError:
            continue
        if r.n_pairs == 0:
            assert line.strip() == ''
            continue
        rec = json.loads(line)
        ok, _ = pf.validate_record(rec)
        assert ok
        x, y, st, anc, desc, t = r.decoded(0)[:6]
        rx, ry, rst, ranc, rdesc, rt = pf.decode_pair(rec)[:6]
        assert np.array_equal(x, rx) and np.array_equal(y, ry) and st == rst and anc == ranc and desc == rdesc
        assert t == rt
