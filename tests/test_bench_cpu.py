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
