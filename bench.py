"""Benchmark of the batched 2D pair-HMM E-step on GB300.

Default workload: MixDom2 with n_dom=3, n_frag=1, n_classes=1 (17 states),
200 pairs with ancestor lengths LogUniform(30, 600), per-pair t, forward +
backward + expected counts -- one E-step over the batch per step (synthetic
data, seed 0 + rank).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

metric: cell-state updates per second of the E-step, where one E-step over a
pair counts (Lx+1)(Ly+1)*N cell-state updates (real lengths, no padding).
`value` times the persistent batched launch with inputs resident in HBM;
`e2e` times the public API call (pairhmm.api.estep_batch_mixdom2) from host
sequences to host results, host<->device copies included.  L2 is flushed
(256 MiB write) between timed steps.  Multi-GPU runs are independent
replicas (pairs are independent; no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, 'tkf-mixdom_gb300')
for _p in (ROOT, PKG_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)

WORKLOAD = 'mixdom2_k3f1c1_200pairs_len30-600'
# per workload: what one step runs and what the metric counts
WORKLOADS = {
    'mixdom2_k3f1c1_200pairs_len30-600': {
        'forward_only': False, 'metric': 'pair-HMM E-step cell-state updates/s',
        'model': 'MixDom2 n_dom=3 n_frag=1 n_classes=1', 'e2e_api': 'pairhmm.api.estep_batch_mixdom2'},
    'mixdom2_k4f2c2_32pairs_len200-1500': {
        'forward_only': False, 'metric': 'pair-HMM E-step cell-state updates/s',
        'model': 'MixDom2 n_dom=4 n_frag=2 n_classes=2',
        'e2e_api': 'pairhmm.api.mixdom2_log_prob(...).sum().backward() (gradient of the summed LL)'},
    'mixdom2_k8f4c4_64pairs_len2000': {
        'forward_only': False, 'metric': 'pair-HMM E-step cell-state updates/s',
        'model': 'MixDom2 n_dom=8 n_frag=4 n_classes=4', 'e2e_api': 'pairhmm.api.estep_batch_mixdom2'},
    'tkf91_64pairs_len50-150': {
        'forward_only': True, 'metric': 'pair-HMM forward cell-state updates/s',
        'model': 'TKF91', 'e2e_api': 'pairhmm.api.estep_batch_tkf92_forward_only (ext = 0)'},
}
# DRAM bytes per launch of each kernel on each workload, from the committed ncu
# captures (profiles/traffic.json; the Markdown summaries beside it give the commands)
TRAFFIC_FILE = os.path.join(ROOT, 'profiles', 'traffic.json')
SMS = 152
FP32_LANES_PER_SM = 128


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--workload', default=WORKLOAD)
    ap.add_argument('--no-plain', action='store_true')
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--pairs', type=int, default=0,
                    help='use only the first P pairs (small case for ncu captures)')
    ap.add_argument('--variant', type=int, default=0,
                    help='kernel family (phmm_set_variant; 0 = automatic)')
    ap.add_argument('--max-len', type=int, default=0,
                    help='truncate every sequence to at most L residues (small case for ncu captures)')
    ap.add_argument('--cpu-seconds', type=float, default=12.0)
    ap.add_argument('--no-tune', action='store_true', help='skip the autotuner (library defaults)')
    ap.add_argument('--dense', action='store_true',
                    help='give the kernels only the dense chi (no factored MixDom transitions)')
    ap.add_argument('--no-accuracy', action='store_true',
                    help='skip the accuracy leg (every pair against the FP64 oracle)')
    ap.add_argument('--serving-requests', type=int, default=2000,
                    help='requests in the serving-stream leg (0: skip it)')
    ap.add_argument('--serving-rate', type=float, default=5000.0)
    ap.add_argument('--tensor', action='store_true',
                    help='wide kernels: forward contraction on the tensor cores as 3xTF32 (phmm_tuning.tensor)')
    ap.add_argument('--banded-pairs', type=int, default=1024,
                    help='pairs of the banded-vs-full E-step leg (0: skip)')
    return ap.parse_args()


def dist_setup(args):
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rank, local


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return json.load(f), 'measured'
    except OSError:
        return {'hbm_gbs': 6800.0, 'bf16_tflops': 1900.0, 'sm_max_mhz': 2070.0}, 'fallback'


def hbm_roofline(kernel, n_states, total_cells, dur_ms, hbm_peak_gbs, traffic):
    """The dominant kernel against the HBM roofline.  Algorithmic bytes: the
    lattice records the kernel must write (a wavefront) or read (the count
    pass, both lattices) or both (a fused forward + backward): per cell and
    lattice one float per emitting state (n_states - 2: S and E emit nothing)
    and one exponent."""
    lattices = 2 if ('count' in kernel or 'fwdbwd' in kernel) else 1
    bpc = lattices * (n_states - 1) * 4
    achieved = bpc * total_cells / (dur_ms / 1e3) / 1e9
    return {'bound': 'hbm', 'kernel': kernel, 'achieved': achieved, 'peak': hbm_peak_gbs, 'unit': 'GB/s',
            'frac': achieved / hbm_peak_gbs, 'traffic': traffic, 'bytes_per_cell': bpc}


def profile_traffic(workload, kernel):
    """DRAM bytes per launch of `kernel` on `workload` from profiles/traffic.json
    (None when no capture covers it)."""
    try:
        with open(TRAFFIC_FILE) as f:
            return float(json.load(f)[workload][kernel.split('::')[-1]])
    except (OSError, ValueError, KeyError, TypeError):
        return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', f'--id={self.gpu_id}', f'--query-gpu={self.Q}',
                 '--format=csv,noheader,nounits', '-lms', '100'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.6)

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in out.strip().splitlines():
            f = [v.strip() for v in line.split(',')]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith('active'):
                    reasons.add(n)
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': mx,
                'reasons': sorted(reasons), 'samples': len(sm)}


def _oracle_model(workload, b):
    """(chi, state types, groups, EM, EI, ED) of pair b under the oracle."""
    from oracle import estep as oe
    p = dict(workload.params)
    p['t'] = float(workload.ts[b])
    if workload.model == 'mixdom2':
        return oe.mixdom2_model(p)[:6]
    return oe.tkf_model(workload.model, p)[:6]


def _oracle_engine():
    """'C' when the oracle's C half (oracle/fb2d.c, built by build()) loads,
    else 'NumPy'."""
    try:
        from oracle import cdp
        if cdp.available():
            cdp._lib()
            return 'C'
    except Exception:
        pass
    return 'NumPy'


def _oracle_pair(workload, b, forward_only):
    """Oracle log-likelihood and expected transition counts (None when forward only)."""
    from oracle import models as om, dp as odp
    chi, st, groups, EM, EI, ED = _oracle_model(workload, b)
    emit = odp.log_emission_table(st, groups, workload.xs[b], workload.ys[b], EM, EI, ED)
    if _oracle_engine() == 'C':
        from oracle import cdp
        return cdp.forward_backward(om.safe_log(chi), st, emit, forward_only)
    if forward_only:
        return odp.forward_table(om.safe_log(chi), st, emit)[0], None
    ll, _, n, _, _ = odp.forward_backward(om.safe_log(chi), st, emit)
    return ll, n


def cpu_baseline(workload, seconds, forward_only, threads=1):
    """The FP64 oracle on a bounded sample of the same pairs (host cores),
    smallest pairs first."""
    done_cells = 0
    t0 = time.perf_counter()
    order = np.argsort(workload.cells())
    n = 0
    N = workload.n_states
    truncated = None
    try:
        from oracle import cdp
        if cdp.available():
            cdp.set_threads(threads)
    except Exception:
        pass
    for b in order:
        cells_b = (len(workload.xs[b]) + 1) * (len(workload.ys[b]) + 1)
        if n == 0 and cells_b * N * N > 2e9:
            # one pair alone is far beyond the time budget: time its leading
            # a x a block (x[:a], y[:a]), a sized from a 16 x 16 calibration run
            sub = lambda a: _leading_block(workload, b, a)
            tc = time.perf_counter()
            _oracle_pair(sub(16), 0, forward_only)
            per_cell = (time.perf_counter() - tc) / 17 ** 2
            a = int(max(16, min(len(workload.xs[b]), (seconds / per_cell) ** 0.5 - 1)))
            t0 = time.perf_counter()
            _oracle_pair(sub(a), 0, forward_only)
            done_cells += (a + 1) * (a + 1)
            n += 1
            truncated = a
            break
        _oracle_pair(workload, b, forward_only)
        done_cells += cells_b
        n += 1
        if time.perf_counter() - t0 > seconds:
            break
    el = time.perf_counter() - t0
    what = 'forward' if forward_only else 'forward+backward+counts'
    smp = (f'{n} smallest pairs of the workload ({done_cells} cells)' if truncated is None else
           f'the leading {truncated} x {truncated} block of the smallest pair ({done_cells} cells)')
    eng = _oracle_engine()
    return {'value': done_cells * N / el, 'unit': 'cell-state updates/s', 'cores': threads,
            'kind': 'port', 'sample': f'{smp}, FP64 {eng} oracle {what}, {el:.1f} s'}


def _leading_block(workload, b, a):
    """Pair b of the workload cut to its leading a x a block (x[:a], y[:a])."""
    from pairhmm.synth import Workload
    return Workload(workload.name, workload.model, workload.params, [workload.xs[b][:a]],
                    [workload.ys[b][:a]], workload.ts[b:b + 1], workload.K, workload.F, workload.C)


def accuracy_leg(workload, gpu, forward_only, block=None, sample_pairs=None):
    """Error of the GPU outputs against the FP64 C oracle over EVERY pair of the
    workload (all host cores, one single-threaded oracle process per core,
    largest pairs first), outside the timed region.  gpu: host arrays 'll'
    (and 'n_trans', 'cnt_M', 'cnt_I', 'cnt_D') indexed like the workload.
    block / sample_pairs: the workload is a sub-sample (the pairs' leading
    blocks, run on the GPU as their own batch) -- said in the result."""
    from oracle import pool
    if _oracle_engine() != 'C':
        return {'error': 'the C oracle is not built (build())'}
    cores = len(os.sched_getaffinity(0))
    P = len(workload.xs)
    cases = [tuple(_oracle_model(workload, b)) + (workload.xs[b], workload.ys[b]) for b in range(P)]
    t0 = time.perf_counter()
    res = pool.estep_pairs(cases, forward_only, cores)
    el = time.perf_counter() - t0
    ll_err, n_abs, n_rel, c_abs, c_rel = [], [], [], [], []
    for b, (ll, n, cnt) in enumerate(res):
        ll_err.append(abs(float(gpu['ll'][b]) - ll) / max(abs(ll), 1e-300))
        if n is None:
            continue
        a, r = pool.count_errors(gpu['n_trans'][b], n)
        n_abs.append(a)
        n_rel.append(r)
        for key, want in zip(('cnt_M', 'cnt_I', 'cnt_D'), cnt):
            a, r = pool.count_errors(gpu[key][b], want)
            c_abs.append(a)
            c_rel.append(r)
    cells = int(sum((len(x) + 1) * (len(y) + 1) for x, y in zip(workload.xs, workload.ys)))
    acc = {'pairs': P, 'cells': cells,
           'max_pair': [int(max(len(x) for x in workload.xs)), int(max(len(y) for y in workload.ys))],
           'll_max_rel_err': float(np.max(ll_err)), 'll_median_rel_err': float(np.median(ll_err)),
           'against': 'FP64 C oracle (oracle/fb2d.c, pinned to the reference outputs)',
           'oracle_s': round(el, 1), 'oracle_cores': cores}
    if n_abs:
        acc.update({'n_trans_max_err_of_max': float(np.max(n_abs)), 'n_trans_max_rel_err': float(np.max(n_rel)),
                    'counts_max_err_of_max': float(np.max(c_abs)), 'counts_max_rel_err': float(np.max(c_rel)),
                    'counts_rel_err_note': 'relative error over entries above 1e-6 of the pair\'s largest'})
    acc['scope'] = ('every pair of the workload' if block is None else
                    f'leading {block} x {block} blocks of {sample_pairs} pairs, run on the GPU as their own batch')
    return acc


def _ref_worker(args):
    sys.path[:0] = [ROOT, PKG_DIR]
    workload, b, forward_only = args
    _oracle_pair(workload, b, forward_only)
    return (len(workload.xs[b]) + 1) * (len(workload.ys[b]) + 1)


def run_reference(args, rank, ws):
    """CPU arm: the reference's algorithm (FP64 restatement) on all host cores."""
    if rank != 0:
        return
    import multiprocessing as mp
    from pairhmm import synth
    w = synth.CONFIGS[args.workload](seed=0)
    cores = len(os.sched_getaffinity(0))
    fwd_only = WORKLOADS[args.workload]['forward_only']
    from pairhmm.synth import Workload
    N = w.n_states
    # bounded sample with the workload's length mix: every stride-th pair in
    # size order, about 2 s of oracle work per core per step; a pair longer
    # than c on a side is timed on its leading block (at most c x c), so no
    # task exceeds half a core's share of a step and the pool stays balanced
    # cell-state updates per core per step (the oracle's cost per cell-state
    # grows with N: ~2.8 M/s per core at 17 states, forward only ~3x that)
    per_core = 5e6 * 17.0 / N * (3.0 if fwd_only else 1.0)
    c = max(8, int((per_core / 2 / N) ** 0.5) - 1)
    clipped = lambda b: (min(len(w.xs[b]), c), min(len(w.ys[b]), c))
    work = lambda b: (clipped(b)[0] + 1) * (clipped(b)[1] + 1) * N
    order = sorted(range(len(w.xs)), key=work, reverse=True)      # largest first
    stride = max(1, int(np.ceil(sum(work(b) for b in order) / (per_core * cores))))
    sample, cells = [], 0
    for b in order[::stride]:
        lx, ly = clipped(b)
        one = Workload(w.name, w.model, w.params, [w.xs[b][:lx]], [w.ys[b][:ly]], w.ts[b:b + 1], w.K, w.F, w.C)
        sample.append((one, 0, fwd_only))
        cells += (lx + 1) * (ly + 1)
    # one process per core: keep each worker's BLAS to one thread (the
    # workers inherit this environment), or they oversubscribe the cores
    for var in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ.setdefault(var, '1')
    ctx = mp.get_context('spawn')
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_worker, sample[-cores:], chunksize=1)
        t0 = time.perf_counter()
        tot = 0
        for _ in range(args.steps):
            tot += sum(pool.imap_unordered(_ref_worker, sample, chunksize=1))
        el = time.perf_counter() - t0
    N = w.n_states
    val = tot * N / el
    line = {'metric': WORKLOADS[args.workload]['metric'], 'value': val, 'unit': 'cell-state updates/s',
            'impl': 'reference', 'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': el / args.steps * 1e3, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': args.workload, 'sample_pairs': len(sample), 'sample_cells': int(cells),
                       'note': 'reference is JAX-only (not installable here); its algorithm is run '
                               f'as the FP64 {_oracle_engine()} restatement in oracle/'},
            'cpu_baseline': {'value': val, 'unit': 'cell-state updates/s', 'cores': cores, 'kind': 'port',
                             'sample': f'{len(sample)} pairs (every {stride}. in size order; sides above {c} '
                                       f'clipped to their leading block), {int(cells)} cells per step'},
            'e2e': {'value': val, 'unit': 'cell-state updates/s', 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line))


def serving_leg(n_requests, rate, seed=0):
    """The serving stream: Poisson arrivals of single-pair E-step requests,
    models mixed uniformly over TKF92 / MixDom2 K*F=3 / MixDom2 K*F=8,
    ancestor lengths LogUniform(20, 2000); continuous batching against
    one-launch-per-request, on the same arrival times."""
    import torch
    from pairhmm import synth
    from pairhmm.serving import Request, Server, ServedModel, latency_summary, run_stream
    t0 = time.perf_counter()
    models, reqs, offsets = synth.make_serving_stream(n_requests, rate=rate, seed=seed)
    gen_s = time.perf_counter() - t0
    served = [ServedModel(name, kind, p) for name, (kind, p) in models.items()]
    ARENA = 48 << 30   # HBM arena of the request loop (workspaces, inputs, outputs)
    n_states = {'tkf92': 5, 'mixdom2_k3f1c1': 17, 'mixdom2_k4f2c2': 42}
    cs = float(sum((len(x) + 1) * (len(y) + 1) * n_states[m] for m, x, y, _ in reqs))

    def one(max_inflight, max_batch):
        srv = Server(served, arena_bytes=ARENA, max_inflight=max_inflight, max_batch=max_batch)
        warm = [Request(-1 - i, m, x, y, t) for i, (m, x, y, t) in enumerate(reqs[:12])]
        for r in warm:
            srv.submit(r)
        srv.drain()
        torch.cuda.synchronize()
        rs = [Request(i, m, x, y, t) for i, (m, x, y, t) in enumerate(reqs)]
        out, wall = run_stream(srv.sched, rs, offsets)
        summ = latency_summary(out, wall)
        summ['cell_states_per_s'] = cs / wall
        summ['batches'] = srv.sched.batches
        summ['mean_batch'] = float(np.mean(srv.sched.batch_sizes)) if srv.sched.batch_sizes else 0.0
        summ['peak_arena_bytes'] = int(srv.sched.peak_bytes)
        return summ
    cont = one(max_inflight=8, max_batch=64)
    plain = one(max_inflight=1, max_batch=1)
    # the same requests offered below saturation (arrival times stretched), so
    # the latency of the batching itself shows apart from queueing
    below = {}
    base_offsets = offsets
    for r in (1000.0, 2000.0, 3000.0):
        if r >= rate:
            continue
        offsets = np.asarray(base_offsets) * (rate / r)
        summ = one(max_inflight=8, max_batch=64)
        below[f'{r:g}'] = {k: summ[k] for k in ('p50_ms', 'p99_ms', 'mean_ms', 'req_per_s', 'failed', 'mean_batch')}
    offsets = base_offsets
    return {'workload': f'Poisson {rate:g} req/s, {n_requests} requests, model uniform over TKF92 (5) / '
                        'MixDom2 K3F1C1 (17) / MixDom2 K4F2C2 (42), ancestor LogUniform(20,2000)',
            'arrival_span_s': float(offsets[-1]), 'cell_states': cs,
            'continuous': cont, 'plain_one_launch_per_request': plain,
            'continuous_below_saturation': below,
            'arena_bytes': ARENA, 'stream_generation_s': gen_s}


def banded_leg(n_pairs, length=500, band=32, reps=7, seed=0):
    """The banded E-step (phmm_estep_band: the reference's
    forward_backward_2d_banded, dp/hmm.py:2395-2491, over a batch) against the
    full-lattice E-step of the same pairs: TKF91 pairs of about
    length x length, band of half-width `band` around the diagonal.  The
    stripes skip the anti-diagonal steps off their rows' band, so the time
    should follow the band's cells, not the lattice's."""
    import torch
    from pairhmm import _lib, api, synth
    from pairhmm import models as pm
    rng = np.random.default_rng(seed)
    Q, pi, _ = synth.rand_Q_pi(rng)
    t = 0.5
    chi = pm.tkf91_trans(0.03, 0.035, t).numpy()
    st = np.array([0, 1, 2, 3, 4], np.int8)
    sub = pm.transition_matrix(pm._t(Q), t).numpy()
    lens = [(int(length * rng.uniform(0.95, 1.05)), int(length * rng.uniform(0.95, 1.05))) for _ in range(n_pairs)]
    xs = [rng.integers(0, 20, a) for a, _ in lens]
    ys = [rng.integers(0, 20, b) for _, b in lens]
    centers = [np.round(np.arange(a + 1) * b / a).astype(int) for a, b in lens]
    W = api.pad_to_bin(band)
    masks = [api.band_mask(a, b, c, band) for (a, b), c in zip(lens, centers)]
    EM, EI, ED = api._tkf_tables(sub, pi)
    plan = api.get_plan(st, np.zeros(5, np.int32), EM.shape[0])
    mk = lambda m: _lib.make_batch(xs, ys, chi[None], np.asarray(EM)[None], np.asarray(EI)[None],
                                   np.asarray(ED)[None], device='cuda', cell_masks=m)
    bb, bf = mk(masks), mk(None)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device='cuda')

    def timed(fn):
        for _ in range(3):
            out = fn()
        torch.cuda.synchronize()
        ts = []
        for k in range(reps):
            flush.fill_(k & 0xff)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts)), out
    band_ms, ob = timed(lambda: _lib.estep_band(plan, bb, centers, W))
    full_ms, of = timed(lambda: _lib.estep(plan, bf))
    band_cells = int(sum(int(m.astype(bool).sum()) for m in masks))
    full_cells = int(sum((a + 1) * (b + 1) for a, b in lens))
    llb, llf = ob['ll'].cpu().numpy(), of['ll'].cpu().numpy()
    return {'workload': f'TKF91, {n_pairs} pairs of about {length} x {length}, band half-width {W} '
                        'around the diagonal', 'api': 'phmm_estep_band (pairhmm.api.estep_batch_banded)',
            'band_cells': band_cells, 'full_cells': full_cells, 'band_ms': band_ms, 'full_ms': full_ms,
            'speedup': full_ms / band_ms, 'cell_ratio': full_cells / band_cells,
            'band_cell_states_per_s': band_cells * 5 / (band_ms / 1e3),
            'status_nonzero': int((ob['status'] != 0).sum().item()),
            'band_ll_below_full': bool(np.all(llb <= llf + 1e-9 * np.abs(llf)))}


def accuracy_of_workload(args, w, plan, out, chi, EM, EI, ED, fwd_only, dev):
    """The accuracy leg of this run: every pair against the oracle, except for
    lattices the oracle cannot finish in about a minute (162 states at 2000 x
    2000): those are checked on the leading block of two pairs, the GPU
    running the same blocks as a batch of their own."""
    import torch
    from pairhmm import _lib
    N = w.n_states
    if float(w.cells().sum()) * N * N <= 1.5e11:
        gpu = {k: v.cpu().numpy() for k, v in out.items()}
        return accuracy_leg(w, gpu, fwd_only)
    a = 1000 if N * N * 1001 * 1001 <= 3e10 else 400
    pick = [int(i) for i in np.argsort(w.cells())[:2]]
    from pairhmm.synth import Workload
    sub = Workload(w.name, w.model, w.params, [w.xs[b][:a] for b in pick], [w.ys[b][:a] for b in pick],
                   np.asarray(w.ts)[pick], w.K, w.F, w.C)
    idx = torch.as_tensor(pick, device=dev)
    bt = _lib.make_batch(sub.xs, sub.ys, chi[idx], EM[idx], EI[idx], ED[idx], device=dev)
    if fwd_only:
        ll, st = _lib.forward(plan, bt)
        gpu = {'ll': ll.cpu().numpy()}
    else:
        gpu = {k: v.cpu().numpy() for k, v in _lib.estep(plan, bt).items()}
    return accuracy_leg(sub, gpu, fwd_only, block=a, sample_pairs=len(pick))


def e2e_function(workload, w, api, torch):
    """The public call a user makes for this workload, host inputs to host outputs."""
    if workload == 'tkf91_64pairs_len50-150':
        Lx = np.array([len(x) for x in w.xs])
        Ly = np.array([len(y) for y in w.ys])
        xp = np.zeros((len(w.xs), Lx.max()), np.int64)
        yp = np.zeros((len(w.ys), Ly.max()), np.int64)
        for b, (x, y) in enumerate(zip(w.xs, w.ys)):
            xp[b, :len(x)] = x
            yp[b, :len(y)] = y
        p = w.params
        return lambda: {'log_p': api.estep_batch_tkf92_forward_only(
            xp, yp, w.ts, Lx, Ly, p['ins_rate'], p['del_rate'], 0.0, p['Q'], p['pi']).cpu().numpy()}
    if workload == 'mixdom2_k4f2c2_32pairs_len200-1500':
        names = ['main_ins', 'main_del', 'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates',
                 'class_pis', 'class_S_exch', 'classdist']

        def grad_call():
            tens = {k: torch.tensor(np.asarray(w.params[k], float), dtype=torch.float64, requires_grad=True)
                    for k in names}
            tt = torch.tensor(np.asarray(w.ts, float), dtype=torch.float64, requires_grad=True)
            ll = api.mixdom2_log_prob(tens['main_ins'], tens['main_del'], tt, tens['dom_ins'], tens['dom_del'],
                                      tens['dom_weights'], tens['frag_weights'], tens['ext_rates'],
                                      tens['class_pis'], tens['class_S_exch'], tens['classdist'], w.xs, w.ys)
            ll.sum().backward()
            out = {k: v.grad.numpy() for k, v in tens.items()}
            out['t'] = tt.grad.numpy()
            out['log_p'] = ll.detach().cpu().numpy()
            return out
        return grad_call
    return lambda: api.to_host(api.estep_batch_mixdom2(w.params, w.xs, w.ys, w.ts))


def main():
    args = parse_args()
    ws, rank, local = dist_setup(args)
    if args.impl == 'reference':
        return run_reference(args, rank, ws)
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group('nccl', device_id=torch.device('cuda', local))
    from pairhmm import synth, api, _lib
    from pairhmm import models as pm
    dev = torch.device('cuda', local)
    w = synth.CONFIGS[args.workload](seed=0)
    shard = None
    if ws > 1:
        # one combined workload of ws x the configuration (seeds 0..ws-1), split
        # over the ranks by longest-processing-time packing of the E-step cost:
        # every rank holds about one configuration's work (weak scaling)
        from pairhmm import replicas
        parts = [w] + [synth.CONFIGS[args.workload](seed=s) for s in range(1, ws)]
        allx = [x for q in parts for x in q.xs]
        ally = [y for q in parts for y in q.ys]
        allt = np.concatenate([np.asarray(q.ts) for q in parts])
        shard = replicas.lpt_partition(replicas.pair_costs(allx, ally, w.n_states), ws)[rank]
        w.xs = [allx[i] for i in shard]
        w.ys = [ally[i] for i in shard]
        w.ts = allt[shard]
    if args.pairs:
        w.xs, w.ys, w.ts = w.xs[:args.pairs], w.ys[:args.pairs], w.ts[:args.pairs]
    if args.max_len:
        w.xs = [x[:args.max_len] for x in w.xs]
        w.ys = [y[:args.max_len] for y in w.ys]
    spec = WORKLOADS[args.workload]
    fwd_only = spec['forward_only']
    N = w.n_states
    cells = w.cells()
    cell_states = float((cells * N).sum())
    # ---- inputs resident in HBM
    if w.model == 'mixdom2':
        K, F, chi, csubs, EM, EI, ED = api._mixdom2_tables(w.params, w.ts, dev)
        plan = api.get_plan(pm.mixdom_state_types(K, F), pm.mixdom_state_groups(K, F), K * F)
    else:
        tt = torch.as_tensor(np.asarray(w.ts, np.float64), device=dev)
        chi = pm.tkf91_trans(w.params['ins_rate'], w.params['del_rate'], tt.cpu()).to(dev)
        EM, EI, ED = pm.tables_tkf(pm.transition_matrix(pm._t(w.params['Q'], dev), tt), pm._t(w.params['pi'], dev))
        plan = api.get_plan(np.array([pm.S, pm.M, pm.I, pm.D, pm.E]), np.zeros(5, np.int32), 1)
    nest, nest_kf = None, None
    if w.model == 'mixdom2' and not args.dense:   # the factored MixDom transitions (phmm_batch.nest)
        nest, nest_kf = api._mixdom2_nest(w.params, w.ts, dev), (K, F)
    batch = _lib.make_batch(w.xs, w.ys, chi, EM, EI, ED, device=dev, nest=nest, nest_kf=nest_kf)
    if args.variant:
        plan.set_variant(args.variant)
    if args.tensor:   # the wide kernels' forward contraction on the tensor cores (3xTF32)
        plan.set_tuning(**dict(plan.get_tuning(), tensor=1))
    # the project's autotuner (pairhmm.autotune) picks the launch configuration
    # for this batch before anything is timed; skipped when one call is long
    tuning = None
    if not args.no_tune and not args.variant and not args.tensor:
        from pairhmm import autotune
        t0 = time.perf_counter()
        (_lib.forward(plan, batch) if fwd_only else _lib.estep(plan, batch))
        torch.cuda.synchronize()
        one_ms = (time.perf_counter() - t0) * 1e3
        if one_ms < 200.0:
            r = autotune.tune(plan, batch, forward_only=fwd_only)
            tuning = {'chosen': r['tuning'], 'ms': r['ms'], 'default_ms': r['default_ms'],
                      'evaluated': r['evaluated'], 'by': 'pairhmm.autotune (coordinate descent, CUDA events)'}
        else:
            tuning = {'chosen': plan.get_tuning(), 'skipped': f'one call takes {one_ms:.0f} ms'}
    plan.set_timing(True)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(out):
        if fwd_only:
            ll, st = _lib.forward(plan, batch)
            return {'ll': ll, 'status': st}
        return _lib.estep(plan, batch, out=out)
    out = None
    for _ in range(max(3, args.warmup)):
        out = step(out)
    torch.cuda.synchronize()
    launches_per_step = plan.launches
    status = out['status'].cpu().numpy()
    try:
        gid = str(torch.cuda.get_device_properties(dev).uuid)
        gid = gid if gid.startswith('GPU-') else f'GPU-{gid}'
    except Exception:
        gid = str(local)
    sampler = ClockSampler(gid)
    sampler.start()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    step_ms, fwd_ms, bwd_ms, cnt_ms = [], [], [], []
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = step(out)
        e1.record(stream)
        a, b = plan.kernel_times()
        fwd_ms.append(a)
        bwd_ms.append(b)
        cnt_ms.append(plan.kernel_time(2))
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clocks = sampler.stop()
    total_ms = float(np.sum(step_ms))
    cells_all = cell_states   # cell-state updates of one step over all ranks (each rank its LPT shard)
    if ws > 1:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        c = torch.tensor([cell_states], device=dev, dtype=torch.float64)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
        cells_all = float(c.item())
    value = cells_all * args.steps / (total_ms / 1e3)
    ms_step = total_ms / args.steps
    # ---- end to end through the public API (host sequences -> host results)
    e2e_ms = []
    h2d = int(sum(len(x) + len(y) for x, y in zip(w.xs, w.ys)) + 8 * len(w.ts))
    d2h = 0
    e2e_call = e2e_function(args.workload, w, api, torch)
    for k in range(0 if args.no_e2e else args.warmup + args.steps):
        flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host = e2e_call()
        t1 = time.perf_counter()
        if k >= args.warmup:
            e2e_ms.append((t1 - t0) * 1e3)
        d2h = int(sum(v.nbytes for v in host.values()))
    e2e_total = float(np.sum(e2e_ms)) if e2e_ms else float('nan')
    if ws > 1:
        t = torch.tensor([e2e_total], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = cells_all * args.steps / (e2e_total / 1e3)
    # ---- plain: one launch sequence per pair (the single-pair path)
    plain = None
    if not args.no_plain and rank == 0 and not fwd_only:
        subs = []
        for b in range(len(w.xs)):
            subs.append(_lib.make_batch([w.xs[b]], [w.ys[b]], chi[b:b + 1], EM[b:b + 1],
                                        EI[b:b + 1], ED[b:b + 1], device=dev))
        plan.set_timing(False)
        for sb in subs[:3]:
            _lib.estep(plan, sb)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for sb in subs:
            _lib.estep(plan, sb)
        e1.record(stream)
        e1.synchronize()
        pms = e0.elapsed_time(e1)
        plain = {'value': cell_states / (pms / 1e3), 'ms_per_step': pms,
                 'pairs_per_s': len(w.xs) / (pms / 1e3),
                 'note': 'same pairs, one phmm_estep call (forward + backward launch) per pair'}
    # ---- roofline of the dominant kernel
    peaks, src = measured_peaks()
    fwd_avg, bwd_avg, cnt_avg = float(np.mean(fwd_ms)), float(np.mean(bwd_ms)), float(np.mean(cnt_ms))
    total_cells = float(cells.sum())
    # the kernels contract through the factored record only for the layouts the library has
    nest_used = (nest is not None and bool(_lib.load().phmm_nest_supported(*nest_kf))
                 and plan.last_variant in (6, 7))
    # (kernel name, algorithmic FLOP per cell) of forward, backward, count pass
    fam = {1: (('forward_kernel', 2), ('backward_kernel', 4), (None, 0)),
           2: (('warp2::forward_warp_kernel', 2), ('warp2::backward_warp_kernel', 4), (None, 0)),
           3: (('blk::forward_block_kernel', 2), ('blk::backward_block_kernel', 4), (None, 0)),
           4: (('warp2::forward_warp_kernel', 2), ('warp2::backward_rec_warp_kernel', 2),
               ('warp2::count_warp_kernel', 2)),
           5: (('blk::fwdbwd_block_kernel', 4), (None, 0), ('blk::count_block_kernel', 2)),
           6: ((('wide::wide_nest_kernel', 2 if fwd_only else 4) if nest_used else
                (('wide::forward_wide_kernel', 2) if fwd_only else ('wide::fwdbwd_wide_kernel', 4))), (None, 0),
               ('wide::count_wide_kernel', 2)),
           7: (('warp2::stripe_tw_kernel<...,0>', 2), ('warp2::stripe_tw_kernel<...,1>', 2),
               ('warp2::count_tw_kernel', 2))}[plan.last_variant]
    durs = [fwd_avg, bwd_avg, cnt_avg]
    # the overlapped count pass (variants 4, 7) starts with the wavefronts and waits
    # on their progress, so its event span is not its own duration
    overlapped = plan.last_variant in (4, 7)
    di = int(np.argmax(durs[:2] if overlapped else durs))
    dom, fpc = fam[di]
    flop = fpc * N * N * total_cells
    dur = durs[di]
    achieved = flop / (dur / 1e3) / 1e12
    fp32_peak = SMS * FP32_LANES_PER_SM * 2 * peaks.get('sm_max_mhz', 2070.0) * 1e6 / 1e12
    roofline = {'bound': 'fp32', 'kernel': dom, 'achieved': achieved, 'peak': fp32_peak,
                'unit': 'TFLOP/s', 'frac': achieved / fp32_peak,
                'traffic': profile_traffic(args.workload, dom),
                'peak_source': f'{SMS} SMs x {FP32_LANES_PER_SM} FP32 lanes x 2 FLOP x sm_max_mhz '
                               f'({peaks.get("sm_max_mhz")} MHz, {src} MEASURED_PEAKS.json); '
                               'the DP is a dense FP32 CUDA-core contraction: no tensor-core or HBM bound',
                'flop_per_cell': fpc * N * N,
                'flop_accounting': ('dense 2N^2 per cell per pass; with the factored MixDom transitions '
                                    '(config.transitions) this is effective FLOP: the factored recursions '
                                    'execute about 5 (5KF) + 11 K F^2 (forward) and 4 (5KF) + 11 K F^2 '
                                    '(backward) multiply-adds per cell (two-warp, K=3 F=1: 108 and 93 against '
                                    '240; wide, K=8 F=4: about 3 (5KF) + 11 K F^2 = 1,888 against 26,880)'
                                    if nest_used
                                    else 'dense 2N^2 per cell per pass'),
                'fwd_kernel_ms': fwd_avg, 'bwd_kernel_ms': bwd_avg, 'count_kernel_ms': cnt_avg,
                'count_overlaps_wavefronts': overlapped,
                'kernels': [f[0] for f in fam if f[0]],
                'hbm_peak_gbs': peaks.get('hbm_gbs')}
    try:   # the same kernel seen against HBM (the DP moves little data: a low fraction is expected)
        roofline_hbm = hbm_roofline(dom, N, total_cells, dur, float(peaks.get('hbm_gbs') or 6800.0),
                                    roofline['traffic'])
    except Exception as e:   # never lose the bench line to this extra view
        roofline_hbm = {'error': repr(e)}
    serving = None
    if rank == 0 and args.serving_requests > 0 and args.workload == WORKLOAD:
        serving = serving_leg(args.serving_requests, args.serving_rate)
    banded = None
    if rank == 0 and args.banded_pairs > 0 and args.workload == WORKLOAD:
        try:
            banded = banded_leg(args.banded_pairs)
        except Exception as e:   # never lose the bench line to this extra leg
            banded = {'error': repr(e)}
    if rank == 0:
        cpu = cpu_baseline(w, args.cpu_seconds, fwd_only) if args.cpu_seconds > 0 else None
        acc = None
        if not args.no_accuracy:
            try:
                acc = accuracy_of_workload(args, w, plan, out, chi, EM, EI, ED, fwd_only, dev)
            except Exception as e:   # never lose the bench line to the oracle leg
                acc = {'error': repr(e)}
        line = {
            'metric': spec['metric'], 'value': value,
            'unit': 'cell-state updates/s', 'n_gpus': ws, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': ms_step, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': args.workload, 'model': spec['model'],
                       'n_states': N, 'pairs_per_gpu': len(w.xs), 'cells_per_gpu': int(total_cells),
                       'cell_states_per_step_per_gpu': cell_states, 'pairs_per_s': len(w.xs) * ws / (ms_step / 1e3),
                       'l2': 'flushed (256 MiB write) between timed steps',
                       'parallelism': (f'replicas x{ws}, one combined workload of {ws} configurations '
                                       'LPT-sharded by E-step cost' if ws > 1 else 'replicas x1'),
                       'tuning': tuning,
                       'wide_contraction': '3xTF32 tensor cores' if args.tensor else 'float32 CUDA cores',
                       'transitions': ('factored MixDom chi (phmm_batch.nest)' if nest_used
                                       else 'dense chi'),
                       'status_nonzero': int((status != 0).sum())},
            'roofline': roofline, 'roofline_hbm': roofline_hbm, 'cpu_baseline': cpu, 'accuracy': acc,
            'e2e': {'value': e2e_value, 'unit': 'cell-state updates/s', 'h2d_bytes_per_step': h2d,
                    'd2h_bytes_per_step': d2h, 'ms_per_step': e2e_total / args.steps,
                    'api': spec['e2e_api']},
            'plain': plain, 'serving': serving, 'banded': banded, 'gpu_launches': launches_per_step * args.steps, 'clocks': clocks,
        }
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
