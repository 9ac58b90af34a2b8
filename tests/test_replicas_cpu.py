"""Multi-GPU host logic (pairhmm.replicas) on the CPU: the LPT split of pairs
over ranks, and a world_size-2 gloo run whose gathered per-pair outputs and
float64 totals equal a single-process run.  The per-rank E-step here is the
oracle (the GPU kernels are covered by the gpu-marked tests)."""
import os
import socket

import numpy as np
import pytest

from pairhmm.replicas import estep_sharded, lpt_partition, pair_costs, partition_loads


def test_lpt_covers_every_pair_once_and_balances():
    rng = np.random.default_rng(0)
    costs = np.exp(rng.uniform(np.log(30), np.log(600), 200)) ** 2
    for n in (1, 2, 3, 8):
        parts = lpt_partition(costs, n)
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(200))
        loads = partition_loads(costs, parts)
        # LPT bound: makespan <= 4/3 OPT, and OPT >= max(mean load, largest item)
        opt_lb = max(costs.sum() / n, costs.max())
        assert loads.max() <= 4.0 / 3.0 * opt_lb + 1e-6


def test_lpt_small_cases():
    assert [p.tolist() for p in lpt_partition([5, 1, 1, 1, 1, 1], 2)] == [[0], [1, 2, 3, 4, 5]]
    parts = lpt_partition([3, 3, 2, 2, 2], 2)
    assert sorted(partition_loads([3, 3, 2, 2, 2], parts).tolist()) == [5.0, 7.0]
    assert [p.tolist() for p in lpt_partition([], 3)] == [[], [], []]


def _workload():
    rng = np.random.default_rng(11)
    from pairhmm import synth
    p = synth.mixdom2_params(rng, 1, 1, 1)
    xs = [rng.integers(0, 20, int(rng.integers(3, 14))) for _ in range(7)]
    ys = [rng.integers(0, 20, int(rng.integers(3, 14))) for _ in range(7)]
    ts = np.exp(rng.uniform(np.log(0.1), np.log(1.5), 7))
    return p, xs, ys, ts


def _oracle_local(p):
    def fn(xs, ys, ts):
        from oracle import estep as oe
        ll, nt = [], []
        for x, y, t in zip(xs, ys, ts):
            a, n, _ = oe.e_step_mixdom2(dict(p, t=float(t)), x, y)
            ll.append(a)
            nt.append(n)
        N = 7
        return {'log_p': np.array(ll, dtype=np.float64),
                'n_trans': np.array(nt, dtype=np.float64).reshape(len(xs), N, N)}
    return fn


def _worker(rank, ws, port, out_dir):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=ws)
    try:
        p, xs, ys, ts = _workload()
        per_pair, totals, idx = estep_sharded(xs, ys, ts, 7, _oracle_local(p))
        np.savez(os.path.join(out_dir, f'rank{rank}.npz'), idx=idx, **{f'pp_{k}': v for k, v in per_pair.items()},
                 **{f'tot_{k}': v for k, v in totals.items()})
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_gloo_two_ranks_equal_single_process(tmp_path):
    import torch.multiprocessing as mp
    ws = 2
    mp.start_processes(_worker, args=(ws, _free_port(), str(tmp_path)), nprocs=ws, join=True,
                       start_method='spawn')
    p, xs, ys, ts = _workload()
    want = _oracle_local(p)(xs, ys, ts)
    idx_all = []
    for r in range(ws):
        d = np.load(tmp_path / f'rank{r}.npz')
        idx_all.append(d['idx'])
        np.testing.assert_allclose(d['pp_log_p'], want['log_p'], rtol=1e-12)
        np.testing.assert_allclose(d['pp_n_trans'], want['n_trans'], rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(d['tot_log_p'], want['log_p'].sum(), rtol=1e-12)
        np.testing.assert_allclose(d['tot_n_trans'], want['n_trans'].sum(axis=0), rtol=1e-12, atol=1e-15)
    assert np.array_equal(np.sort(np.concatenate(idx_all)), np.arange(len(xs)))
    assert all(len(i) > 0 for i in idx_all)
    # the split follows the E-step cost
    parts = lpt_partition(pair_costs(xs, ys, 7), ws)
    assert all(np.array_equal(a, b) for a, b in zip(idx_all, parts))
