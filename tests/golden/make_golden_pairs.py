"""Golden fixtures for the precompiled X/A/Y pair records, produced by the
reference's own ``util/pair_format.py``: records of seeded random pairs and
alignments written by ``encode_pair`` (one JSON line each, as the shards hold
them once decompressed), their ``decode_pair`` outputs, and the
``validate_record`` verdicts of a few broken records.

Usage (needs the reference checkout; writes tests/golden/pairs.jsonl and
tests/golden/pairs.npz):

    python tests/golden/make_golden_pairs.py <reference>/python
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import jax_shim  # noqa: E402


def main(ref_python):
    jax_shim.install()
    sys.path.insert(0, ref_python)
    from tkfmixdom.jax.util import pair_format as ref
    rng = np.random.default_rng(20261208)
    lines, out = [], {}
    for p in range(12):
        Lx, Ly = (int(v) for v in rng.integers(1, 60, 2))
        if p == 0:
            Lx, Ly = 1, 1
        n_m = int(rng.integers(0, min(Lx, Ly) + 1))
        states = np.array([1] * n_m + [3] * (Lx - n_m) + [2] * (Ly - n_m))
        rng.shuffle(states)
        anc = rng.integers(0, 20, Lx)
        desc = rng.integers(0, 20, Ly)
        t = float(rng.uniform(0.01, 3.0))
        fam = f'PF{int(rng.integers(0, 99999)):05d}'
        kw = {}
        if p % 3 == 1:
            kw['gamma_labels'] = [int(v) for v in rng.integers(-1, 4, len(states))]
        if p % 4 == 2:
            kw['gamma_log_posteriors'] = rng.normal(size=(4, len(states))).tolist()
        rec = ref.encode_pair(anc.tolist(), desc.tolist(), states.tolist(), t, fam, f'r{p}a', f'r{p}b', **kw)
        lines.append(json.dumps(rec))
        x_int, y_int, st, ac, dc, t_est, _, _ = ref.decode_pair(rec)
        pre = f'p{p}_'
        out[pre + 'anc_in'] = anc
        out[pre + 'desc_in'] = desc
        out[pre + 'states_in'] = states
        out[pre + 't_in'] = np.float64(t)
        out[pre + 'fam'] = np.array(fam)
        out[pre + 'x_int'] = np.asarray(x_int)
        out[pre + 'y_int'] = np.asarray(y_int)
        out[pre + 'states'] = np.asarray(st, np.int64)
        out[pre + 'anc_chars'] = np.asarray(ac, np.int64)
        out[pre + 'desc_chars'] = np.asarray(dc, np.int64)
        out[pre + 't_est'] = np.float64(t_est)
    bad = [{'x': 'ACD', 'a': 'M2', 'y': 'AC', 't': 0.1}, {'x': 'AC', 'a': 'M2I1', 'y': 'AC', 't': 0.1},
           {'x': 'ABC', 'a': 'M3', 'y': 'ACD', 't': 0.1}, {'x': 'ACD', 'a': 'M3', 'y': 'ACZ', 't': 0.1}]
    for k, rec in enumerate(bad):
        ok, msg = ref.validate_record(rec)
        out[f'bad{k}_record'] = np.array(json.dumps(rec))
        out[f'bad{k}_ok'] = np.bool_(ok)
        out[f'bad{k}_msg'] = np.array(msg)
    out['n_pairs'] = np.int64(len(lines))
    with open(os.path.join(HERE, 'pairs.jsonl'), 'w') as f:
        f.write('\n'.join(lines) + '\n')
    np.savez_compressed(os.path.join(HERE, 'pairs.npz'), **out)
    print('wrote', len(lines), 'records')


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden_pairs.py <reference checkout>/python')
    main(sys.argv[1])
