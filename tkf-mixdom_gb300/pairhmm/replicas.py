"""Pairs across GPUs: replicas with no collective on the data path.

Pairs are independent (the reference vmaps over them with shared
parameters, train/tkf92_svi_bw.py:214-217), so a multi-GPU E-step is one
batch per rank and a host-side reduction afterwards, as the reference's own
training script sums per-pair results on the host (train_pfam.py:2858-2876):

* ``lpt_partition`` splits pairs over ranks by longest-processing-time bin
  packing of the E-step cost (Lx+1)(Ly+1)N^2 (the per-rank step time is the
  largest per-rank cost, so the ranks finish together);
* each rank runs its shard through the batched E-step on its own GPU;
* ``gather_pairs`` returns every pair's outputs to every rank in the
  caller's order, and ``reduce_totals`` sums count totals in float64.

The exchange is one all_gather of host objects after the step (gloo or any
backend with object collectives); nothing runs between GPUs while the DP
kernels run.
"""
from __future__ import annotations

import heapq

import numpy as np


def pair_costs(xs, ys, n_states):
    """E-step cost of each pair: (Lx+1)(Ly+1) N^2."""
    return np.array([(len(x) + 1) * (len(y) + 1) for x, y in zip(xs, ys)], dtype=np.float64) * n_states ** 2


def lpt_partition(costs, n_ranks):
    """Longest-processing-time bin packing: pairs in decreasing cost, each to
    the rank with the least load so far (ties: lowest rank).  Returns one
    sorted index array per rank."""
    costs = np.asarray(costs, dtype=np.float64)
    heap = [(0.0, r) for r in range(n_ranks)]
    parts = [[] for _ in range(n_ranks)]
    for i in np.argsort(-costs, kind='stable'):
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def partition_loads(costs, parts):
    costs = np.asarray(costs, dtype=np.float64)
    return np.array([costs[p].sum() for p in parts])


def _world(group):
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def gather_pairs(local, indices, n_pairs, group=None):
    """All ranks' per-pair outputs back in the caller's pair order.

    local: dict of arrays with the rank's pairs on axis 0 (host numpy);
    indices: the rank's pair indices.  Returns a dict of [n_pairs, ...]
    float64/int arrays on every rank."""
    import torch.distributed as dist
    rank, ws = _world(group)
    mine = {k: np.asarray(v) for k, v in local.items()}
    if ws == 1:
        items = [(np.asarray(indices), mine)]
    else:
        items = [None] * ws
        dist.all_gather_object(items, (np.asarray(indices), mine), group=group)
    keys = mine.keys()
    out = {}
    for k in keys:
        proto = next(d[k] for _, d in items if d[k].shape[0] > 0) if any(d[k].shape[0] for _, d in items) \
            else mine[k]
        arr = np.zeros((n_pairs,) + proto.shape[1:], dtype=proto.dtype)
        for idx, d in items:
            if len(idx):
                arr[idx] = d[k]
        out[k] = arr
    return out


def reduce_totals(totals, group=None):
    """Float64 sum of per-rank count totals (dict of arrays) on every rank."""
    import torch
    import torch.distributed as dist
    rank, ws = _world(group)
    out = {}
    for k in sorted(totals):
        t = torch.as_tensor(np.asarray(totals[k], dtype=np.float64))
        if ws > 1:
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        out[k] = t.numpy()
    return out


def estep_sharded(xs, ys, ts, n_states, local_fn, group=None):
    """Run an E-step over pairs split across the ranks of `group`.

    local_fn(xs, ys, ts) -> dict of per-pair host arrays for the rank's
    shard (e.g. ``pairhmm.api.estep_batch_mixdom2`` with its outputs copied
    to the host).  Returns (per-pair outputs of all pairs, totals summed over
    pairs, this rank's indices)."""
    rank, ws = _world(group)
    parts = lpt_partition(pair_costs(xs, ys, n_states), ws)
    idx = parts[rank]
    local = local_fn([xs[i] for i in idx], [ys[i] for i in idx], np.asarray(ts)[idx])
    local = {k: np.asarray(v) for k, v in local.items()}
    per_pair = gather_pairs(local, idx, len(xs), group)
    sums = {k: v.sum(axis=0) for k, v in local.items()
            if k not in ('status',) and np.issubdtype(v.dtype, np.floating)}
    totals = reduce_totals(sums, group)
    return per_pair, totals, idx
