"""Captured CUDA graphs of the batched MixDom2 E-step (estep_batch_mixdom2).

The reference compiles one XLA program per padded batch shape and reuses it
(its per-shape jit cache, train_pfam.py:1674-1741).  Here the kernels are
fixed, and what a call costs beyond them is the host side: packing parameters
and residues, planning the work lists, and issuing about twenty launches,
copies and stream joins.  For a batch shape seen before -- the same model
shape and the same pair lengths, as in every EM iteration over one set of
pairs -- the whole device sequence is replayed from a CUDA graph captured
once:

  pinned host blocks -> device   (parameter block, Holmes-Rubin class blocks,
                                  residues, per-pair times)
  phmm_mixdom2_tables[_nest]_dp  (chi, P_c(t), emission tables; chi's factored
                                  form where the kernels use it)
  phmm_estep_ws_launch           (the split E-step on a graph-owned workspace
                                  whose work description was written once)
  phmm_mixdom2_class_counts_dp   (per-class counts)
  phmm_holmes_rubin_dp           (class_W, class_U)

A call then fills the pinned blocks (parameters packed by the library, the
class eigendecompositions from its cache), replays the graph on the caller's
stream and returns the outputs as fresh device tensors (one device-to-device
copy of the output arena), so results of earlier calls stay valid.  The
parameters, residues and times may change from call to call; only the model
shape and the lengths are frozen into a graph.
"""
from __future__ import annotations

import ctypes
import os
import warnings
from collections import OrderedDict

import numpy as np
import torch

from . import _lib
from . import models as pm

_GRAPHS = OrderedDict()
_SEEN = {}
MAX_GRAPHS = 2          # graph-owned workspaces are lattice-sized: keep few
CAPTURE_AFTER = 2       # capture on the second call with a batch shape


def enabled():
    return os.environ.get('PAIRHMM_GRAPHS', '1') != '0'


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class MixDom2EStepGraph:
    """One batch shape (K, F, C and the pair lengths) of estep_batch_mixdom2
    with class counts, captured as a CUDA graph on `device`."""

    def __init__(self, pro, xs, ys, device):
        self.lib = _lib.load()
        self.dev = torch.device(device)
        K, F, C, A = pro.K, pro.F, pro.C, pro.A
        self.K, self.F, self.C, self.A = K, F, C, A
        buf, xo, yo, Lx, Ly = _lib.pack_residues(xs, ys)
        self.Lx, self.Ly = Lx, Ly
        self.total = int(Lx.sum() + Ly.sum())
        P = self.P = int(Lx.size)
        N, G = 2 + 5 * K * F, K * F
        pin = lambda n, dt: torch.empty(n, dtype=dt, pin_memory=True)
        dev = lambda n, dt: torch.empty(n, dtype=dt, device=self.dev)
        nb = int(self.lib.phmm_mixdom2_param_block_bytes())
        nh = int(self.lib.phmm_holmes_rubin_block_bytes(C))
        # pinned host inputs and their device copies
        self.h_par, self.d_par = pin(nb, torch.uint8), dev(nb, torch.uint8)
        self.h_hr, self.d_hr = pin(nh, torch.uint8), dev(nh, torch.uint8)
        self.h_res, self.d_res = pin(buf.size, torch.uint8), dev(buf.size, torch.uint8)
        self.h_t, self.d_t = pin(P, torch.float64), dev(P, torch.float64)
        # prologue outputs
        f32, f64 = torch.float32, torch.float64
        self.chi = torch.empty(P, N, N, dtype=f32, device=self.dev)
        self.EM = torch.empty(P, G, 21, 21, dtype=f32, device=self.dev)
        self.EI = torch.empty(P, G, 21, dtype=f32, device=self.dev)
        self.ED = torch.empty(P, G, 21, dtype=f32, device=self.dev)
        self.csubs = torch.empty(P, C, A, A, dtype=f64, device=self.dev)
        # the factored transitions, where the kernels have them for (K, F)
        self.nest = (torch.empty(P, 20 * K * F + 25 * K * F * F, dtype=f32, device=self.dev)
                     if pro.nest_supported() else None)
        # outputs in one arena
        self.specs = [('ll', (P,), f64), ('n_trans', (P, N, N), f64), ('cnt_M', (P, G, 21, 21), f64),
                      ('cnt_I', (P, G, 21), f64), ('cnt_D', (P, G, 21), f64), ('status', (P,), torch.int32)]
        self.specs += [(k, sh, f64) for k, sh in pro.class_count_shapes(P).items()]
        self.specs += [('class_W', (P, C, A), f64), ('class_U', (P, C, A, A), f64)]
        self.arena = _lib.OutputArena(self.dev, self.specs)
        # the plan (own: its side streams belong to the capture stream) and workspace
        self.plan = _lib.Plan(pm.mixdom_state_types(K, F), pm.mixdom_state_groups(K, F), G)
        self.batch = _lib.DeviceBatch(Lx=Lx, Ly=Ly, x_off=xo, y_off=yo, residues=self.d_res, chi=self.chi,
                                      emit_M=self.EM, emit_I=self.EI, emit_D=self.ED, nest=self.nest,
                                      nest_kf=(K, F))
        need = ctypes.c_size_t()
        _lib._check(self.lib.phmm_workspace_bytes(self.plan.handle, ctypes.byref(self.batch.struct()), 1,
                                                  ctypes.byref(need)), 'phmm_workspace_bytes')
        self.ws = torch.empty(max(int(need.value), 256), dtype=torch.uint8, device=self.dev)
        self.graph = None
        self.stream = torch.cuda.Stream(device=self.dev)
        self.done = torch.cuda.Event()
        self.done_valid = False

    def tune_from(self, plan):
        """Use the launch configuration of another plan of the same state space."""
        self.plan.set_tuning(**plan.get_tuning())

    def _fill(self, pro, xs, ys, ts):
        if self.done_valid:
            self.done.synchronize()   # the previous replay has read the pinned blocks
        _lib._check(self.lib.phmm_mixdom2_param_block(ctypes.byref(pro.struct), ctypes.c_void_p(self.h_par.data_ptr()),
                                                      self.h_par.numel()), 'phmm_mixdom2_param_block')
        Q = pro.class_Q()
        pis = np.ascontiguousarray(pro._arr['class_pis'])
        _lib._check(self.lib.phmm_holmes_rubin_block(self.C, self.A, Q.ctypes.data, pis.ctypes.data,
                                                     ctypes.c_void_p(self.h_hr.data_ptr()), self.h_hr.numel()),
                    'phmm_holmes_rubin_block')
        # residues in pack_residues's layout (x_0, y_0, x_1, y_1, ...), checked as there
        parts = [None] * (2 * len(xs))
        parts[0::2] = xs
        parts[1::2] = ys
        allr = np.concatenate(parts) if parts else np.zeros(0, np.int64)
        if allr.ndim != 1:
            raise ValueError('sequences must be one-dimensional')
        if allr.size != self.total or (allr.size and (allr.min() < 0 or allr.max() > 20)):
            raise ValueError('residues must be integers in 0..20 (20 = wildcard), with the captured lengths')
        self.h_res.numpy()[:allr.size] = allr
        if isinstance(ts, torch.Tensor):
            self.h_t.copy_(ts.detach().reshape(-1).to(torch.float64).cpu())
        else:
            self.h_t.numpy()[:] = np.asarray(ts, np.float64).reshape(-1)

    def _sequence(self, stream):
        """The device work of one call, issued on `stream` (eager or captured)."""
        s = ctypes.c_void_p(stream.cuda_stream)
        lib, P = self.lib, self.P
        with torch.cuda.stream(stream):
            self.d_par.copy_(self.h_par, non_blocking=True)
            self.d_hr.copy_(self.h_hr, non_blocking=True)
            self.d_res.copy_(self.h_res, non_blocking=True)
            self.d_t.copy_(self.h_t, non_blocking=True)
        if self.nest is not None:   # the tables and the factored record from one build of chi
            _lib._check(lib.phmm_mixdom2_tables_nest_dp(_ptr(self.d_par), self.K, self.F, self.C, P, _ptr(self.d_t),
                                                        _ptr(self.chi), _ptr(self.EM), _ptr(self.EI), _ptr(self.ED),
                                                        _ptr(self.csubs), _ptr(self.nest), s),
                        'phmm_mixdom2_tables_nest_dp')
        else:
            _lib._check(lib.phmm_mixdom2_tables_dp(_ptr(self.d_par), self.K, self.F, self.C, P, _ptr(self.d_t),
                                                   _ptr(self.chi), _ptr(self.EM), _ptr(self.EI), _ptr(self.ED),
                                                   _ptr(self.csubs), s), 'phmm_mixdom2_tables_dp')
        ar = self.arena
        _lib._check(lib.phmm_estep_ws_launch(self.plan.handle, ctypes.byref(self.batch.struct()), _ptr(self.ws),
                                             self.ws.numel(), _ptr(ar['ll']), _ptr(ar['n_trans']), _ptr(ar['cnt_M']),
                                             _ptr(ar['cnt_I']), _ptr(ar['cnt_D']), _ptr(ar['status']), s),
                    'phmm_estep_ws_launch')
        _lib._check(lib.phmm_mixdom2_class_counts_dp(
            _ptr(self.d_par), self.K, self.F, self.C, P, _ptr(self.csubs), _ptr(ar['cnt_M']), _ptr(ar['cnt_I']),
            _ptr(ar['cnt_D']), _ptr(ar['class_match_counts']), _ptr(ar['class_insert_counts']),
            _ptr(ar['class_delete_counts']), _ptr(ar['classdist_counts']), s), 'phmm_mixdom2_class_counts_dp')
        _lib._check(lib.phmm_holmes_rubin_dp(_ptr(self.d_hr), self.C, P, _ptr(self.d_t),
                                             _ptr(ar['class_match_counts']), _ptr(ar['class_W']),
                                             _ptr(ar['class_U']), s), 'phmm_holmes_rubin_dp')

    def capture(self, pro, xs, ys, ts):
        """Write the work description, run the sequence once eagerly on the
        capture stream (side streams, kernel attributes), then capture it."""
        self._fill(pro, xs, ys, ts)
        cur = torch.cuda.current_stream(self.dev)
        self.stream.wait_stream(cur)
        _lib._check(self.lib.phmm_estep_ws_prepare(self.plan.handle, ctypes.byref(self.batch.struct()),
                                                   _ptr(self.ws), self.ws.numel(),
                                                   ctypes.c_void_p(self.stream.cuda_stream)), 'phmm_estep_ws_prepare')
        self._sequence(self.stream)
        self.stream.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.stream, capture_error_mode='thread_local'):
            self._sequence(self.stream)
        self.graph = g
        cur.wait_stream(self.stream)

    def __call__(self, pro, xs, ys, ts):
        """Outputs of one call as fresh device tensors (the keys of
        estep_batch_mixdom2 with class counts)."""
        self._fill(pro, xs, ys, ts)
        cur = torch.cuda.current_stream(self.dev)
        self.stream.wait_stream(cur)
        with torch.cuda.stream(self.stream):
            self.graph.replay()
            buf = self.arena.buf.clone()
        self.done.record(self.stream)
        self.done_valid = True
        cur.wait_stream(self.stream)
        buf.record_stream(cur)
        return _lib.arena_views(buf, self.arena.layout)


def _key(pro, xs, ys):
    Lx = np.fromiter(map(len, xs), np.int64, len(xs))
    Ly = np.fromiter(map(len, ys), np.int64, len(ys))
    return (pro.K, pro.F, pro.C, pro.A, Lx.tobytes(), Ly.tobytes())


def mixdom2_estep(pro, xs, ys, ts, device, tuned_plan=None):
    """The outputs of the batched MixDom2 E-step with class counts from a
    graph of this batch shape, or None when the caller should run it eagerly
    (graphs disabled, a shape not seen CAPTURE_AFTER times, or a failed
    capture: that shape then stays eager)."""
    if not enabled() or pro.C > 8 or pro.A != 20 or pro.K * pro.F > 33 or len(xs) == 0:
        return None
    key = _key(pro, xs, ys)
    g = _GRAPHS.get(key)
    if g is None:
        n = _SEEN.get(key, 0) + 1
        _SEEN[key] = n
        if n < CAPTURE_AFTER or n < 0:
            return None
        try:
            g = MixDom2EStepGraph(pro, xs, ys, device)
            if tuned_plan is not None:
                g.tune_from(tuned_plan)
            g.capture(pro, xs, ys, ts)
        except Exception as e:
            _SEEN[key] = -(1 << 30)   # never again for this shape
            torch.cuda.synchronize()
            warnings.warn(f'CUDA graph capture of the batched E-step failed ({e!r}); this batch shape runs '
                          'eagerly', RuntimeWarning)
            return None
        _GRAPHS[key] = g
        while len(_GRAPHS) > MAX_GRAPHS:
            _GRAPHS.popitem(last=False)
    else:
        _GRAPHS.move_to_end(key)
    return g(pro, xs, ys, ts)


def clear():
    """Drop every captured graph (and its device memory)."""
    _GRAPHS.clear()
    _SEEN.clear()
