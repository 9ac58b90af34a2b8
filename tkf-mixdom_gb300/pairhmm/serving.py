"""Continuous-batching request loop for pair-HMM E-step jobs.

Requests are single pairs ``(model, x, y, t)``; each asks for the pair's
log-likelihood and its Baum-Welch expected counts (``n_trans`` and the
per-group character counts; for MixDom2 also the per-class counts of
``e_step_mixdom2``, train/likelihood.py:279-344).  The reference has no
serving loop: its callers run one bucketed ``jit(vmap(forward_backward_2d))``
per padded shape (train_pfam.py:1674-1741, 2672-2907).  Here:

* models are registered once; their parameters and a plan per state space
  stay on the device;
* every batch's device memory (kernel workspace, inputs, outputs) is carved
  from one HBM arena; a batch is admitted only when its bytes fit in the
  arena's free space, so admission is memory-based and exact;
* up to ``max_inflight`` batches run at once, each on its own CUDA stream, so
  a request that arrives while others are on the GPU is launched as soon as
  a stream and memory are free and its kernels overlap theirs (continuous
  batching, not a queue in front of one launch at a time);
* a batch is the oldest queued request plus the queued requests of the same
  model behind it, in arrival order, up to ``max_batch`` requests and the
  free memory;
* results are read back into pinned host memory and a batch retires when
  its CUDA event has completed; ``poll()`` never blocks.

The policy (``Scheduler``) is separate from the device work (``Executor``)
so it runs on the CPU against a fake executor in the tests.
"""
from __future__ import annotations

import bisect
import time
from dataclasses import dataclass, field

import numpy as np

ALIGN = 256


def _al(n):
    return (int(n) + ALIGN - 1) // ALIGN * ALIGN


@dataclass
class Request:
    """One pair-HMM E-step job."""
    rid: int
    model: str
    x: np.ndarray
    y: np.ndarray
    t: float
    arrival: float = 0.0          # time.perf_counter() when it arrived
    admitted: float | None = None
    done: float | None = None
    result: dict | None = None
    error: str | None = None
    est_bytes: int = 0

    @property
    def latency(self):
        return None if self.done is None else self.done - self.arrival


class Arena:
    """First-fit allocator of 256-byte-aligned ranges inside ``size`` bytes.

    It hands out offsets only; the device buffer behind them belongs to the
    executor.  Free ranges are kept sorted and coalesced."""

    def __init__(self, size):
        self.size = int(size) // ALIGN * ALIGN
        self._free = [(0, self.size)] if self.size else []   # sorted (offset, length)
        self.used = 0

    def alloc(self, nbytes):
        n = _al(max(nbytes, 1))
        for k, (off, ln) in enumerate(self._free):
            if ln >= n:
                if ln == n:
                    del self._free[k]
                else:
                    self._free[k] = (off + n, ln - n)
                self.used += n
                return off, n
        return None

    def release(self, off, n):
        k = bisect.bisect_left(self._free, (off, 0))
        self._free.insert(k, (off, n))
        # coalesce with the neighbours
        if k + 1 < len(self._free) and self._free[k][0] + self._free[k][1] == self._free[k + 1][0]:
            self._free[k] = (off, n + self._free[k + 1][1])
            del self._free[k + 1]
        if k > 0 and self._free[k - 1][0] + self._free[k - 1][1] == self._free[k][0]:
            self._free[k - 1] = (self._free[k - 1][0], self._free[k - 1][1] + self._free[k][1])
            del self._free[k]
        self.used -= n

    def largest_free(self):
        return max((ln for _, ln in self._free), default=0)

    def free_ranges(self):
        return list(self._free)


@dataclass
class _InFlight:
    reqs: list
    off: int
    nbytes: int
    handle: object
    slot: int


class Scheduler:
    """Admission and retirement policy of the request loop.

    ``executor`` provides ``request_bytes(req)`` (an upper bound of the
    device bytes one request adds to a batch), ``batch_bytes(model, reqs)``
    (the exact bytes of that batch), ``launch(model, reqs, off, nbytes, slot)``
    (enqueue the batch, return a handle), ``ready(handle)`` and
    ``finish(handle, reqs)`` (store each request's ``result``)."""

    def __init__(self, executor, arena_bytes, max_inflight=4, max_batch=64, clock=time.perf_counter):
        self.ex = executor
        self.arena = Arena(arena_bytes)
        self.max_inflight = int(max_inflight)
        self.max_batch = int(max_batch)
        self.clock = clock
        self.queue: list[Request] = []
        self.inflight: list[_InFlight] = []
        self._free_slots = list(range(self.max_inflight))
        self.completed: list[Request] = []
        self.batches = 0
        self.batch_sizes = []
        self.peak_bytes = 0

    # ---- public
    def submit(self, req: Request, arrival=None):
        req.arrival = self.clock() if arrival is None else arrival
        req.est_bytes = int(self.ex.request_bytes(req))
        if req.est_bytes > self.arena.size:
            req.error = (f'request needs about {req.est_bytes} bytes of device memory, '
                         f'more than the {self.arena.size}-byte arena')
            req.done = self.clock()
            self.completed.append(req)
            return req
        self.queue.append(req)
        return req

    def poll(self):
        """Retire finished batches, then admit queued requests; returns the
        requests completed by this call."""
        done = self._retire()
        self._admit()
        return done

    def idle(self):
        return not self.queue and not self.inflight

    def drain(self, sleep=0.0):
        out = []
        while not self.idle():
            out += self.poll()
            if sleep:
                time.sleep(sleep)
        return out

    # ---- policy
    def _retire(self):
        done = []
        keep = []
        for b in self.inflight:
            if self.ex.ready(b.handle):
                self.ex.finish(b.handle, b.reqs)
                now = self.clock()
                for r in b.reqs:
                    r.done = now
                done += b.reqs
                self.arena.release(b.off, b.nbytes)
                self._free_slots.append(b.slot)
            else:
                keep.append(b)
        self.inflight = keep
        self.completed += done
        return done

    def _admit(self):
        while self.queue and self._free_slots:
            head = self.queue[0]
            room = self.arena.largest_free()
            if head.est_bytes > room:
                return   # wait for memory; the oldest request goes first
            batch, est = [], 0
            for r in self.queue:
                if len(batch) >= self.max_batch:
                    break
                if r.model != head.model:
                    continue
                if est + r.est_bytes > room:
                    break
                batch.append(r)
                est += r.est_bytes
            need = int(self.ex.batch_bytes(head.model, batch))
            while need > room and len(batch) > 1:
                batch.pop()
                need = int(self.ex.batch_bytes(head.model, batch))
            got = self.arena.alloc(need)
            if got is None:
                return
            off, n = got
            slot = self._free_slots.pop()
            ids = {id(r) for r in batch}
            self.queue = [r for r in self.queue if id(r) not in ids]
            now = self.clock()
            for r in batch:
                r.admitted = now
            try:
                handle = self.ex.launch(head.model, batch, off, n, slot)
            except Exception as e:   # a failed launch fails its requests, not the loop
                self.arena.release(off, n)
                self._free_slots.append(slot)
                for r in batch:
                    r.error = f'launch failed: {e}'
                    r.done = self.clock()
                self.completed += batch
                continue
            self.inflight.append(_InFlight(batch, off, n, handle, slot))
            self.batches += 1
            self.batch_sizes.append(len(batch))
            self.peak_bytes = max(self.peak_bytes, self.arena.used)


# ---------------------------------------------------------------- device executor
@dataclass
class ServedModel:
    """A registered model: kind 'tkf92' (5 states) or 'mixdom2' (2+5KF)."""
    name: str
    kind: str
    params: dict
    class_counts: bool = True
    # filled by the executor
    plan: object = None
    n_states: int = 0
    n_groups: int = 0
    extra: dict = field(default_factory=dict)


class CudaExecutor:
    """Runs admitted batches through phmm_estep_ws on per-slot CUDA streams,
    with every per-batch device buffer carved from one arena tensor."""

    def __init__(self, models, arena_bytes, max_inflight, device='cuda'):
        import torch
        from . import _lib
        from . import models as pm
        self.torch, self._lib, self.pm = torch, _lib, pm
        self.device = torch.device(device)
        _lib.load()
        self.arena = torch.empty(int(arena_bytes) // ALIGN * ALIGN, dtype=torch.uint8, device=self.device)
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(max_inflight)]
        self.models = {}
        for m in models:
            self._register(m)

    # ---- models
    def _register(self, m: ServedModel):
        torch, pm, _lib = self.torch, self.pm, self._lib
        from .api import get_plan
        p = m.params
        if m.kind == 'tkf92':
            st = np.array([pm.S, pm.M, pm.I, pm.D, pm.E], np.int8)
            gr = np.zeros(5, np.int32)
            G = 1
            m.extra = {'prologue': _lib.Tkf92Prologue(p['ins_rate'], p['del_rate'], p.get('ext', 0.0),
                                                      p['Q'], p['pi'])}
        elif m.kind == 'mixdom2':
            K = len(np.asarray(p['dom_ins']))
            F = np.asarray(p['frag_weights']).shape[1]
            st = pm.mixdom_state_types(K, F)
            gr = pm.mixdom_state_groups(K, F)
            G = K * F
            pro = _lib.MixDom2Prologue(p)
            # the factored transitions (phmm_batch.nest) where the kernels have them
            m.extra = {'K': K, 'F': F, 'prologue': pro, 'nest': pro.nest_supported()}
        else:
            raise ValueError(f'unknown model kind {m.kind!r}')
        m.plan = get_plan(st, gr, G)
        m.n_states, m.n_groups = len(st), G
        self.models[m.name] = m

    # ---- sizes
    def _io_sizes(self, m, Lx, Ly):
        """Byte sizes of the per-batch inputs and outputs, in carve order."""
        P, N, G = len(Lx), m.n_states, m.n_groups
        sizes = [('ll', 8 * P), ('n_trans', 8 * P * N * N), ('cnt_M', 8 * P * G * 441),
                 ('cnt_I', 8 * P * G * 21), ('cnt_D', 8 * P * G * 21), ('status', 4 * P),
                 ('residues', max(int(np.sum(Lx) + np.sum(Ly)), 16)), ('chi', 4 * P * N * N),
                 ('emit_M', 4 * P * G * 441), ('emit_I', 4 * P * G * 21), ('emit_D', 4 * P * G * 21)]
        pro = m.extra['prologue']
        if m.kind == 'mixdom2':
            sizes += [('t', 8 * P), ('csubs', 8 * P * pro.C * pro.A * pro.A)]
            if m.extra.get('nest'):
                sizes += [('nest', 4 * P * (20 * pro.K * pro.F + 25 * pro.K * pro.F * pro.F))]
        else:
            sizes += [('t', 8 * P), ('csubs', 8 * P * pro.A * pro.A)]
        return sizes

    def _ws(self, m, Lx, Ly):
        return self._lib.workspace_bytes(m.plan, self._lib.host_batch(Lx, Ly), estep=True)

    def request_bytes(self, r):
        m = self.models[r.model]
        Lx, Ly = [len(r.x)], [len(r.y)]
        return self._ws(m, Lx, Ly) + sum(_al(n) for _, n in self._io_sizes(m, Lx, Ly)) + ALIGN

    def batch_bytes(self, model, reqs):
        m = self.models[model]
        Lx = [len(r.x) for r in reqs]
        Ly = [len(r.y) for r in reqs]
        return _al(self._ws(m, Lx, Ly)) + sum(_al(n) for _, n in self._io_sizes(m, Lx, Ly))

    # ---- device work
    def launch(self, model, reqs, off, nbytes, slot):
        torch, _lib = self.torch, self._lib
        m = self.models[model]
        s = self.streams[slot]
        P = len(reqs)
        buf, xo, yo, Lx, Ly = _lib.pack_residues([r.x for r in reqs], [r.y for r in reqs])
        ws_n = _al(self._ws(m, Lx, Ly))
        views, o = {}, off + ws_n
        for name, n in self._io_sizes(m, Lx, Ly):
            views[name] = self.arena[o:o + n]
            o += _al(n)
        assert o - off <= nbytes
        N, G = m.n_states, m.n_groups
        f64 = lambda v, *sh: v.view(torch.float64).view(P, *sh)
        f32 = lambda v, *sh: v.view(torch.float32).view(P, *sh)
        out = {'ll': views['ll'].view(torch.float64), 'n_trans': f64(views['n_trans'], N, N),
               'cnt_M': f64(views['cnt_M'], G, 21, 21), 'cnt_I': f64(views['cnt_I'], G, 21),
               'cnt_D': f64(views['cnt_D'], G, 21), 'status': views['status'].view(torch.int32)}
        host_res = torch.from_numpy(buf).pin_memory()
        host_t = torch.tensor([float(r.t) for r in reqs], dtype=torch.float64).pin_memory()
        chi_v = f32(views['chi'], N, N)
        eM, eI, eD = f32(views['emit_M'], G, 21, 21), f32(views['emit_I'], G, 21), f32(views['emit_D'], G, 21)
        csubs = None
        with torch.cuda.stream(s):
            res = views['residues'][:buf.size]
            res.copy_(host_res, non_blocking=True)
            # device prologue straight into the arena
            pro = m.extra['prologue']
            t_v = views['t'].view(torch.float64)
            t_v.copy_(host_t, non_blocking=True)
            if m.kind == 'mixdom2':
                csubs = views['csubs'].view(torch.float64).view(P, pro.C, pro.A, pro.A)
            else:
                csubs = views['csubs'].view(torch.float64).view(P, pro.A, pro.A)
            nest = None
            if m.kind == 'mixdom2' and m.extra.get('nest'):
                nest = f32(views['nest'], 20 * pro.K * pro.F + 25 * pro.K * pro.F * pro.F)
            pro.run(t_v, chi_v, eM, eI, eD, csubs, stream=s, **({'nest': nest} if nest is not None else {}))
            chi = EM = EI = ED = None
            batch = _lib.DeviceBatch(Lx=Lx, Ly=Ly, x_off=xo, y_off=yo, residues=res, chi=chi_v,
                                     emit_M=eM, emit_I=eI, emit_D=eD, nest=nest,
                                     nest_kf=(m.extra.get('K', 0), m.extra.get('F', 0)))
            _lib.estep_ws(m.plan, batch, (self.arena.data_ptr() + off, ws_n), stream=s, out=out)
            dev_out = dict(out)
            if m.kind == 'mixdom2' and m.class_counts:
                dev_out.update(m.extra['prologue'].class_counts(csubs, out['cnt_M'], out['cnt_I'], out['cnt_D'],
                                                                stream=s))
            host = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in dev_out.items()}
            for k, v in dev_out.items():
                host[k].copy_(v, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(s)
        # keep the host inputs and the temporaries alive until the batch retires
        return {'event': ev, 'host': host, 'keep': (host_res, host_t, batch, chi, EM, EI, ED, csubs, dev_out)}

    def ready(self, h):
        return h['event'].query()

    def finish(self, h, reqs):
        host = {k: v.numpy() for k, v in h['host'].items()}
        for i, r in enumerate(reqs):
            r.result = {('log_p' if k == 'll' else k): v[i].copy() for k, v in host.items()}
            if int(r.result['status']) != 0:
                r.error = f'kernel status {int(r.result["status"])}'


class Server:
    """The request loop: ``submit`` requests, call ``poll`` (non-blocking)
    until they complete, or ``run_stream`` for timed arrivals."""

    def __init__(self, models, arena_bytes=None, max_inflight=4, max_batch=64, device='cuda'):
        import torch
        if arena_bytes is None:
            free, _ = torch.cuda.mem_get_info(torch.device(device))
            arena_bytes = int(free * 0.5)
        self.executor = CudaExecutor(models, arena_bytes, max_inflight, device)
        self.sched = Scheduler(self.executor, arena_bytes, max_inflight, max_batch)

    def submit(self, req, arrival=None):
        return self.sched.submit(req, arrival)

    def poll(self):
        return self.sched.poll()

    def drain(self):
        return self.sched.drain()


def run_stream(sched, requests, offsets, clock=time.perf_counter, sleep=time.sleep):
    """Feed ``requests`` at ``offsets`` seconds after the start, polling the
    scheduler until every request completes.  Returns (requests, wall seconds)."""
    order = np.argsort(offsets, kind='stable')
    t0 = clock()
    i, n = 0, len(requests)
    while i < n or not sched.idle():
        now = clock() - t0
        while i < n and offsets[order[i]] <= now:
            k = order[i]
            sched.submit(requests[k], arrival=t0 + offsets[k])
            i += 1
        sched.poll()
        if sched.idle() and i < n:
            wait = offsets[order[i]] - (clock() - t0)
            if wait > 0:
                sleep(min(wait, 1e-3))
    return requests, clock() - t0


def latency_summary(requests, wall):
    lat = np.array([r.latency for r in requests if r.error is None], dtype=np.float64)
    ok = lat.size
    return {'requests': len(requests), 'completed': int(ok),
            'failed': int(sum(r.error is not None for r in requests)),
            'p50_ms': float(np.percentile(lat, 50) * 1e3) if ok else None,
            'p99_ms': float(np.percentile(lat, 99) * 1e3) if ok else None,
            'mean_ms': float(lat.mean() * 1e3) if ok else None,
            'req_per_s': float(ok / wall) if wall > 0 else None,
            'wall_s': float(wall)}
