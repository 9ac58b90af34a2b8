"""bench.py's pure helpers on the CPU (its GPU legs run on the GB300)."""
import math
import os
import sys

from conftest import ROOT


def _bench():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    return bench


def test_hbm_roofline_view():
    bench = _bench()
    r = bench.hbm_roofline('warp2::stripe_tw_kernel<...,1>', 17, 10.4e6, 2.0, 6806.5, 6.6e8)
    assert r['bound'] == 'hbm' and r['unit'] == 'GB/s'
    assert r['bytes_per_cell'] == 16 * 4
    assert math.isclose(r['achieved'], 64 * 10.4e6 / 2e-3 / 1e9)
    assert math.isclose(r['frac'], r['achieved'] / 6806.5)
    assert bench.hbm_roofline('warp2::count_tw_kernel', 17, 1.0, 1.0, 1.0, None)['bytes_per_cell'] == 128
    assert bench.hbm_roofline('blk::fwdbwd_block_kernel', 42, 1.0, 1.0, 1.0, None)['bytes_per_cell'] == 2 * 41 * 4


def test_every_workload_names_its_metric_and_api():
    bench = _bench()
    for name, spec in bench.WORKLOADS.items():
        assert {'forward_only', 'metric', 'model', 'e2e_api'} <= set(spec), name
    assert bench.WORKLOAD in bench.WORKLOADS
    assert os.path.exists(os.path.join(ROOT, 'bench.py'))


def test_reference_arm_runs_on_the_cpu():
    """`bench.py --impl reference` needs no GPU: one short run prints the
    contract's line (impl, value, cpu_baseline, e2e with zero copies)."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--workload',
                          'tkf91_64pairs_len50-150', '--steps', '1', '--warmup', '1'],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line['impl'] == 'reference' and line['value'] > 0 and line['unit'] == 'cell-state updates/s'
    assert line['cpu_baseline']['kind'] == 'port' and line['cpu_baseline']['cores'] >= 1
    assert line['e2e']['h2d_bytes_per_step'] == 0 and line['e2e']['d2h_bytes_per_step'] == 0
    assert line['higher_is_better'] is True and line['n_gpus'] >= 1


def test_accuracy_leg_every_pair_and_a_planted_error():
    """bench.py's accuracy leg checks every pair: the oracle's own outputs
    report zero error, and an error planted in one pair's copy is found."""
    import numpy as np
    bench = _bench()
    from oracle import build_oracle, cdp
    build_oracle.build()
    from pairhmm import synth
    w = synth.make_mixdom2_workload('small', 2, 1, 1, 20, ('loguniform', 5, 40), seed=3)
    gpu = {'ll': np.zeros(20), 'n_trans': np.zeros((20, 12, 12)), 'cnt_M': np.zeros((20, 2, 21, 21)),
           'cnt_I': np.zeros((20, 2, 21)), 'cnt_D': np.zeros((20, 2, 21))}
    from oracle import pool
    cases = [tuple(bench._oracle_model(w, b)) + (w.xs[b], w.ys[b]) for b in range(20)]
    for b, (ll, n, (cM, cI, cD)) in enumerate(pool.estep_pairs(cases, cores=2)):
        gpu['ll'][b], gpu['n_trans'][b], gpu['cnt_M'][b], gpu['cnt_I'][b], gpu['cnt_D'][b] = ll, n, cM, cI, cD
    acc = bench.accuracy_leg(w, gpu, False)
    assert acc['pairs'] == 20 and acc['scope'] == 'every pair of the workload'
    assert acc['ll_max_rel_err'] == 0.0 and acc['n_trans_max_rel_err'] == 0.0 and acc['counts_max_rel_err'] == 0.0
    gpu['ll'][7] *= 1 + 3e-6
    gpu['cnt_I'][11] *= 1 + 2e-5
    acc = bench.accuracy_leg(w, gpu, False)
    assert 2e-6 < acc['ll_max_rel_err'] < 4e-6
    assert 1e-5 < acc['counts_max_rel_err'] < 3e-5
