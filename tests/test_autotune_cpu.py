"""The autotuner's host logic on the CPU: batch signatures, the JSON cache
(store in one process, found by the next), and the coordinate descent over
the launch axes against a fake plan whose 'time' is a known function of the
configuration."""
import json

import numpy as np


class FakePlan:
    """Stands in for pairhmm._lib.Plan: records set_tuning calls."""
    _st = np.array([0, 1, 2, 3, 4], np.int8)
    _gr = np.zeros(5, np.int32)
    n_states, n_groups = 5, 1

    def __init__(self, families=(7, 4)):
        self.families = families
        self.cfg = None

    def set_tuning(self, variant=0, wave_per_sm=0, count_per_sm=-1, priorities=0, checkpoint=0, tensor=0):
        from pairhmm import _lib
        if variant not in (0,) + tuple(self.families):
            raise _lib.PairHMMError('no kernels of this family')
        self.cfg = (variant, wave_per_sm, count_per_sm, priorities)
        self.ckpt = checkpoint
        self.tensor = tensor


class FakeBatch:
    def __init__(self, Lx, Ly):
        self.Lx, self.Ly = np.asarray(Lx), np.asarray(Ly)


def test_signature_bins_lengths_and_pair_counts():
    from pairhmm import autotune
    a = autotune.batch_signature([100, 200, 300], [110, 190, 290])
    b = autotune.batch_signature([101, 201, 299], [111, 189, 291])   # same bins
    c = autotune.batch_signature([100, 200, 600], [110, 190, 600])   # longer tail
    d = autotune.batch_signature(list(range(1, 6)), list(range(1, 6)))
    assert a == b and a != c and a.startswith('P4-') and d.startswith('P8-')
    assert autotune.batch_signature([], []) == 'P0'


def test_cache_round_trip(tmp_path, monkeypatch):
    from pairhmm import autotune
    monkeypatch.setenv('PAIRHMM_TUNE_CACHE', str(tmp_path / 'tuning.json'))
    autotune._MEM.clear()
    plan, batch = FakePlan(), FakeBatch([50, 60], [55, 70])
    assert autotune.lookup(plan, batch) is None
    entry = {'tuning': {'variant': 7, 'wave_per_sm': 4, 'count_per_sm': -1, 'priorities': 1, 'checkpoint': 0,
                        'tensor': 0},
             'ms': 2.2,
             'default_ms': 2.3, 'evaluated': 9}
    autotune._store(autotune._key(plan, batch), entry)
    autotune._MEM.clear()   # a new process: only the file remains
    assert autotune.lookup(plan, batch) == entry
    assert autotune.apply_cached(plan, batch) == entry['tuning'] and plan.cfg == (7, 4, -1, 1)
    data = json.load(open(tmp_path / 'tuning.json'))
    assert list(data) == [autotune._key(plan, batch)]


def test_coordinate_descent_finds_the_fast_configuration(monkeypatch, tmp_path):
    from pairhmm import autotune
    monkeypatch.setenv('PAIRHMM_TUNE_CACHE', str(tmp_path / 'tuning.json'))
    autotune._MEM.clear()
    plan, batch = FakePlan(), FakeBatch([100] * 8, [90] * 8)
    # time as a function of the configuration: best at family 7, 3 CTAs/SM, no overlap grid, priorities
    cost = lambda v, w, c, p: 2.0 + 0.3 * (v != 7) + 0.1 * abs((w or 2) - 3) + 0.05 * (c != 0) + 0.05 * (p != 1)
    monkeypatch.setattr(autotune, '_time', lambda pl, b, out, reps, flush, fo: (cost(*pl.cfg), None))
    r = autotune.tune(plan, batch, flush_bytes=0, warmup_s=0)
    assert r['tuning'] == {'variant': 7, 'wave_per_sm': 3, 'count_per_sm': 0, 'priorities': 1, 'checkpoint': 0,
                           'tensor': 0}
    assert plan.cfg == (7, 3, 0, 1)
    assert abs(r['ms'] - 2.0) < 1e-9 and r['default_ms'] > r['ms'] and r['evaluated'] == len(r['table'])
    autotune._MEM.clear()
    assert autotune.lookup(plan, batch)['tuning'] == r['tuning']


def test_winner_confirmed_against_fresh_default_timing(monkeypatch, tmp_path):
    """A default timed slow once (a clock ramp) must not hand the win to a
    configuration that is no faster when both are timed again."""
    from pairhmm import autotune
    monkeypatch.setenv('PAIRHMM_TUNE_CACHE', str(tmp_path / 'tuning.json'))
    autotune._MEM.clear()
    plan, batch = FakePlan(), FakeBatch([100] * 8, [90] * 8)
    calls = []

    def fake_time(pl, b, out, reps, flush, fo):
        calls.append(pl.cfg)
        if len(calls) == 1:
            return 3.0, None                          # the first timing runs at low clocks
        return (1.99 if pl.cfg[1] == 4 else 2.0), None  # wave_per_sm=4 within noise of the rest
    monkeypatch.setattr(autotune, '_time', fake_time)
    r = autotune.tune(plan, batch, flush_bytes=0, warmup_s=0, store=False)
    assert r['tuning'] == autotune.DEFAULT and plan.cfg == (0, 0, -1, 0)
    assert abs(r['ms'] - 2.0) < 1e-9 and abs(r['default_ms'] - 2.0) < 1e-9
