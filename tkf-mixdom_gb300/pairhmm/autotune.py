"""Autotuner of the E-step launch configuration (phmm_tuning).

The reference leaves launch shapes to XLA and caches one compiled program
per padded shape (its per-shape jit cache, train_pfam.py:1674-1741, and the
length buckets of train/tkf92_svi_bw.py:435-464).  Here the kernels are fixed
and what varies is how they share the GPU:

* the kernel family, where more than one fits the state space (split E-step
  on two-warp or one-warp stripes; block kernels; wide kernels);
* resident CTAs per SM of each persistent wavefront grid;
* CTAs per SM of the count grid that runs beside the wavefronts (or none);
* stream priorities (wavefronts first when SM slots free up).

Stripe-edge checkpointing (phmm_tuning.checkpoint) is left at its automatic
setting: it trades arithmetic for memory, and a batch that fits either way
runs faster without it.  The tensor-core contraction (phmm_tuning.tensor)
is left off: it changes the results' rounding, which a launch setting must
not.

Results do not depend on the configuration (the same kernels on the same work
items), only the time does.  The search is a coordinate descent over those
axes, each candidate timed with CUDA events on the caller's own batch (median
of a few repetitions after a warm-up), starting from the library's defaults
and keeping a change only when it is faster by more than 1 %.  The winner is
cached per (state space, batch signature) -- the signature is the pair count
and log-binned length quantiles, so a later batch with the same length law
reuses it -- in memory and in a JSON file (PAIRHMM_TUNE_CACHE, default
~/.cache/pairhmm/tuning.json), so another process skips the search.
"""
from __future__ import annotations

import json
import math
import os
import threading
import time
import zlib

import numpy as np
import torch

from . import _lib

DEFAULT = {'variant': 0, 'wave_per_sm': 0, 'count_per_sm': -1, 'priorities': 0, 'checkpoint': 0, 'tensor': 0}
AXES = ('variant', 'wave_per_sm', 'count_per_sm', 'priorities')
_MEM = {}
_LOCK = threading.Lock()


def cache_path():
    return os.environ.get('PAIRHMM_TUNE_CACHE') or os.path.join(os.path.expanduser('~'), '.cache', 'pairhmm',
                                                                'tuning.json')


def _bin(v, base=1.25):
    """Index of v on a geometric grid of ratio `base` (0 for v <= 1)."""
    return 0 if v <= 1 else int(math.floor(math.log(v) / math.log(base)))


def batch_signature(Lx, Ly):
    """Pair count (next power of two) and log-binned quantiles (50, 90, 100 %)
    of the pairs' anti-diagonal counts Lx + Ly."""
    Lx = np.asarray(Lx, np.int64)
    Ly = np.asarray(Ly, np.int64)
    P = int(Lx.size)
    if P == 0:
        return 'P0'
    d = Lx + Ly
    q = [int(np.quantile(d, f)) for f in (0.5, 0.9)] + [int(d.max())]
    return f'P{1 << max(0, (P - 1).bit_length())}-L' + '.'.join(str(_bin(v)) for v in q)


def plan_key(plan):
    st = ''.join(str(int(v)) for v in plan._st)
    gr = ','.join(str(int(v)) for v in plan._gr)
    return f'N{plan.n_states}-G{plan.n_groups}-{st}-{zlib.crc32(gr.encode()):08x}'


def _key(plan, batch):
    return plan_key(plan) + '|' + batch_signature(batch.Lx, batch.Ly)


def _load_file():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, entry):
    with _LOCK:
        _MEM[key] = entry
        path = cache_path()
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            data = _load_file()
            data[key] = entry
            tmp = f'{path}.{os.getpid()}.tmp'
            with open(tmp, 'w') as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, path)
        except OSError:
            pass   # an unwritable cache only costs a search in the next process


def lookup(plan, batch):
    """The cached configuration for this plan's state space and this batch's
    signature, or None."""
    key = _key(plan, batch)
    with _LOCK:
        if key in _MEM:
            return _MEM[key]
        entry = _load_file().get(key)
        if entry is not None:
            _MEM[key] = entry
        return entry


def apply_cached(plan, batch):
    """Set the cached configuration on the plan if there is one (else leave
    the plan's own).  Returns the configuration applied or None."""
    entry = lookup(plan, batch)
    if entry is None:
        return None
    plan.set_tuning(**entry['tuning'])
    return entry['tuning']


def _time(plan, batch, out, reps, flush, forward_only):
    stream = torch.cuda.current_stream()

    def once(o):
        if forward_only:
            _lib.forward(plan, batch)
            return o
        return _lib.estep(plan, batch, out=o)
    out = once(out)
    torch.cuda.synchronize()
    ts = []
    for k in range(reps):
        if flush is not None:
            flush.fill_(k & 0xff)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = once(out)
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts)), out


def _warm(plan, batch, forward_only, seconds):
    """Run the batch for `seconds` first: an idle GPU starts at low clocks, and
    the first configuration timed would otherwise pay for the ramp."""
    end = time.perf_counter() + seconds
    out = None
    while time.perf_counter() < end:
        if forward_only:
            _lib.forward(plan, batch)
        else:
            out = _lib.estep(plan, batch, out=out)
        torch.cuda.synchronize()


def _axes(plan):
    """Values of each axis that fit this state space (the families are probed:
    set_tuning refuses one without kernels for it)."""
    fams = []
    for v in (7, 4, 5, 6):
        try:
            plan.set_tuning(v, 0, -1, 0, 0, 0)
            fams.append(v)
        except _lib.PairHMMError:
            pass
    plan.set_tuning(**DEFAULT)
    return {'variant': [0] + fams, 'wave_per_sm': [0, 1, 2, 3, 4], 'count_per_sm': [-1, 0, 1, 2],
            'priorities': [0, 1]}


def tune(plan, batch, reps=5, forward_only=False, flush_bytes=256 << 20, store=True, warmup_s=0.5):
    """Search the launch configuration for this batch on this plan, apply the
    fastest and (store=True) cache it.  Returns {'tuning', 'ms', 'default_ms',
    'evaluated', 'key', 'table'}; the table lists every configuration timed.
    The GPU is warmed on the batch for warmup_s seconds first, and the winner
    is timed again against the defaults at the end (it must still be faster
    by more than 1 %), so clock ramps and one-off noise do not pick it."""
    flush = torch.empty(flush_bytes, dtype=torch.uint8, device=batch.residues.device) if flush_bytes else None
    axes = _axes(plan)
    if warmup_s > 0:
        _warm(plan, batch, forward_only, warmup_s)
    table = []
    seen = {}

    def score(cfg):
        k = tuple(cfg[a] for a in AXES + ('checkpoint', 'tensor'))
        if k in seen:
            return seen[k]
        try:
            plan.set_tuning(**cfg)
        except _lib.PairHMMError:
            seen[k] = math.inf
            return math.inf
        ms, _ = _time(plan, batch, None, reps, flush, forward_only)
        seen[k] = ms
        table.append(dict(cfg, ms=round(ms, 4)))
        return ms
    best = dict(DEFAULT)
    best_ms = default_ms = score(best)
    for _ in range(2):   # two sweeps of coordinate descent
        improved = False
        for axis in AXES:
            for v in axes[axis]:
                if v == best[axis]:
                    continue
                cfg = dict(best, **{axis: v})
                ms = score(cfg)
                if ms < best_ms * 0.99:
                    best, best_ms, improved = cfg, ms, True
        if not improved:
            break
    if best != DEFAULT:   # confirm against the defaults with fresh timings
        plan.set_tuning(**DEFAULT)
        default_ms, _ = _time(plan, batch, None, reps, flush, forward_only)
        plan.set_tuning(**best)
        best_ms, _ = _time(plan, batch, None, reps, flush, forward_only)
        if not best_ms < default_ms * 0.99:
            best, best_ms = dict(DEFAULT), default_ms
    plan.set_tuning(**best)
    entry = {'tuning': best, 'ms': round(best_ms, 4), 'default_ms': round(default_ms, 4), 'evaluated': len(table)}
    key = _key(plan, batch)
    if store:
        _store(key, entry)
    return dict(entry, key=key, table=table)
