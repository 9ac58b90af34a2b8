"""The precompiled X/A/Y pair records (util/pair_format.py; the shards of
train_pfam.py:984-1029 PrecompiledPairSource).

``read_records`` parses a whole decompressed shard (JSON lines) in the
library's native reader (``phmm_pairs_count`` / ``phmm_pairs_decode``) into
the batch layout the E-step kernels take -- no per-record Python -- and
``PairRecords`` hands out the kernels' inputs: the residue lists for
``make_batch`` / the batched E-steps, the per-column alignment arrays for the
1D forward-backward, the match positions for the match-aligned E-step.  The
per-record helpers mirror the reference's module (same names, arguments and
errors).  Shards are zstd-compressed in the reference; decompression is the
caller's (no zstd codec in this image).
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import re
from dataclasses import dataclass

import numpy as np

from . import _lib

AMINO_ACIDS = "ACDEFGHIKLMNPQRSTVWY"
AA = len(AMINO_ACIDS)
AA_TO_IDX = {a: i for i, a in enumerate(AMINO_ACIDS)}
IDX_TO_AA = dict(enumerate(AMINO_ACIDS))
M_STATE, I_STATE, D_STATE = 1, 2, 3
_LETTER = {M_STATE: 'M', I_STATE: 'I', D_STATE: 'D'}
_STATE = {v: k for k, v in _LETTER.items()}
_RUN = re.compile(r'([MID])(\d+)')


class PairCounts(ctypes.Structure):
    _fields_ = [('n_pairs', ctypes.c_int32), ('n_residues', ctypes.c_int64), ('n_columns', ctypes.c_int64)]


def _bind(lib):
    if getattr(lib, '_pairs_bound', False):
        return lib
    vp = ctypes.c_void_p
    lib.phmm_pairs_count.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(PairCounts)]
    lib.phmm_pairs_count.restype = ctypes.c_int
    lib.phmm_pairs_decode.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(PairCounts)] + [vp] * 13
    lib.phmm_pairs_decode.restype = ctypes.c_int
    lib._pairs_bound = True
    return lib


@dataclass
class PairRecords:
    """A decoded shard: residues in the batch layout plus the alignments."""
    Lx: np.ndarray          # int32 [P]
    Ly: np.ndarray          # int32 [P]
    x_off: np.ndarray       # int64 [P]
    y_off: np.ndarray       # int64 [P]
    residues: np.ndarray    # uint8 [sum Lx + Ly], pair p as [x_p, y_p]
    t: np.ndarray           # float64 [P]
    n_cols: np.ndarray      # int32 [P]
    col_off: np.ndarray     # int64 [P]
    col_state: np.ndarray   # int8 [sum cols]: 1 M, 2 I, 3 D
    col_anc: np.ndarray     # uint8 [sum cols]: ancestor character, 20 for I columns
    col_desc: np.ndarray    # uint8 [sum cols]: descendant character, 20 for D columns
    fam: list               # family of each record (None without one)

    @property
    def n_pairs(self):
        return int(self.Lx.size)

    def x(self, p):
        return self.residues[self.x_off[p]:self.x_off[p] + self.Lx[p]]

    def y(self, p):
        return self.residues[self.y_off[p]:self.y_off[p] + self.Ly[p]]

    def sequences(self):
        """(xs, ys): per-pair residue arrays for make_batch / the batched E-steps."""
        return [self.x(p) for p in range(self.n_pairs)], [self.y(p) for p in range(self.n_pairs)]

    def columns(self, p):
        """(states, anc, desc) of pair p's alignment columns."""
        s = slice(self.col_off[p], self.col_off[p] + self.n_cols[p])
        return self.col_state[s], self.col_anc[s], self.col_desc[s]

    def alignments(self):
        """(cols, ancs, descs, ts): per-pair column arrays and times, the
        inputs of api.estep_1d_mixdom2."""
        cols, ancs, descs = zip(*(self.columns(p) for p in range(self.n_pairs))) if self.n_pairs else ((), (), ())
        return list(cols), list(ancs), list(descs), self.t.copy()

    def match_positions(self, p):
        """0-based (i, j) of the alignment's M columns (mask_emissions_match_aligned)."""
        st, _, _ = self.columns(p)
        xi = np.cumsum(st != I_STATE) - 1
        yj = np.cumsum(st != D_STATE) - 1
        m = st == M_STATE
        return xi[m].astype(np.int32), yj[m].astype(np.int32)

    def decoded(self, p):
        """decode_pair's tuple for record p: (x_int, y_int, states, anc_chars,
        desc_chars, t_est)."""
        st, anc, desc = self.columns(p)
        return (self.x(p).astype(np.int32), self.y(p).astype(np.int32), [int(v) for v in st],
                [int(v) for v in anc[st != I_STATE]], [int(v) for v in desc[st != D_STATE]], float(self.t[p]))


def read_records(data):
    """Parse JSON-lines pair records (str or bytes, a decompressed shard)."""
    lib = _bind(_lib.load())
    raw = data.encode('utf-8') if isinstance(data, str) else bytes(data)
    cnt = PairCounts()
    _lib._check(lib.phmm_pairs_count(raw, len(raw), ctypes.byref(cnt)), 'phmm_pairs_count')
    P, R, C = cnt.n_pairs, cnt.n_residues, cnt.n_columns
    a = {'Lx': np.zeros(P, np.int32), 'Ly': np.zeros(P, np.int32), 'x_off': np.zeros(P, np.int64),
         'y_off': np.zeros(P, np.int64), 'residues': np.zeros(R, np.uint8), 't': np.zeros(P, np.float64),
         'n_cols': np.zeros(P, np.int32), 'col_off': np.zeros(P, np.int64), 'col_state': np.zeros(C, np.int8),
         'col_anc': np.zeros(C, np.uint8), 'col_desc': np.zeros(C, np.uint8)}
    fam_off = np.zeros(P, np.int64)
    fam_len = np.zeros(P, np.int32)
    ptr = lambda v: ctypes.c_void_p(v.ctypes.data if v.size else 0)
    _lib._check(lib.phmm_pairs_decode(raw, len(raw), ctypes.byref(cnt), *[ptr(a[k]) for k in (
        'Lx', 'Ly', 'x_off', 'y_off', 'residues', 't', 'n_cols', 'col_off', 'col_state', 'col_anc', 'col_desc')],
        ptr(fam_off), ptr(fam_len)), 'phmm_pairs_decode')
    fam = [raw[o:o + n].decode('utf-8') if o >= 0 else None for o, n in zip(fam_off, fam_len)]
    return PairRecords(fam=fam, **a)


# ---------------------------------------------------------------- per-record helpers
def rle_encode(states):
    """M/I/D state codes -> run-length string, e.g. [1, 1, 2] -> 'M2I1'."""
    out = []
    for s in states:
        c = _LETTER[s]
        if out and out[-1][0] == c:
            out[-1][1] += 1
        else:
            out.append([c, 1])
    return ''.join(f'{c}{n}' for c, n in out)


def rle_decode(rle_string):
    """Run-length string -> state codes (letters followed by a count; other
    characters are skipped)."""
    states = []
    for c, n in _RUN.findall(rle_string or ''):
        states.extend([_STATE[c]] * int(n))
    return states


def encode_pair(anc_seq, desc_seq, alignment_states, t_est, family_id, row1_name='', row2_name='',
                gamma_labels=None, gamma_log_posteriors=None):
    """A record dict {'x', 'a', 'y', 't', 'fam', 'id'[, 'gamma', 'gamma_lp']}:
    t rounded to 6 decimals, id the first 16 hex digits of the SHA-256 of
    'family:row1:row2' (util/pair_format.py:90-139)."""
    rec = {'x': ''.join(IDX_TO_AA[int(c)] for c in anc_seq),
           'a': rle_encode(list(alignment_states)),
           'y': ''.join(IDX_TO_AA[int(c)] for c in desc_seq),
           't': round(float(t_est), 6),
           'fam': family_id,
           'id': hashlib.sha256(f'{family_id}:{row1_name}:{row2_name}'.encode()).hexdigest()[:16]}
    if gamma_labels is not None:
        rec['gamma'] = [int(g) for g in gamma_labels]
    if gamma_log_posteriors is not None:
        rec['gamma_lp'] = [[round(float(v), 4) for v in row] for row in gamma_log_posteriors]
    return rec


def decode_pair(record):
    """(x_int, y_int, states, anc_chars, desc_chars, t_est, gamma_labels,
    gamma_lp) of one record dict (util/pair_format.py:142-191)."""
    x = np.array([AA_TO_IDX[c] for c in record['x']], dtype=np.int32)
    y = np.array([AA_TO_IDX[c] for c in record['y']], dtype=np.int32)
    states = rle_decode(record['a'])
    anc, desc, xi, yi = [], [], 0, 0
    for s in states:
        if s != I_STATE:
            anc.append(int(x[xi]))
            xi += 1
        if s != D_STATE:
            desc.append(int(y[yi]))
            yi += 1
    return (x, y, states, anc, desc, float(record['t']), record.get('gamma'), record.get('gamma_lp'))


def validate_record(record):
    """(ok, message) as util/pair_format.py:194-223."""
    try:
        states = rle_decode(record['a'])
        n_m = states.count(M_STATE)
        n_i = states.count(I_STATE)
        n_d = states.count(D_STATE)
        if n_m + n_d != len(record['x']):
            return False, f"M+D={n_m + n_d} != len(X)={len(record['x'])}"
        if n_m + n_i != len(record['y']):
            return False, f"M+I={n_m + n_i} != len(Y)={len(record['y'])}"
        for name in ('x', 'y'):
            for c in record[name]:
                if c not in AA_TO_IDX:
                    return False, f"Invalid AA in {name.upper()}: {c}"
        return True, ''
    except Exception as e:   # the reference reports any failure as a message
        return False, str(e)


def write_records(records):
    """JSON lines of record dicts (the shard text before compression)."""
    return ''.join(json.dumps(r) + '\n' for r in records)
