"""ctypes binding of the C ABI in include/pairhmm.h.

This is the only place the Python host touches the CUDA library.  Every
compute call goes through ``libpairhmm.so``; when the library is missing the
calls raise instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np
import torch

from .build import LIB_PATH

_LIB = None

EXPORTS = ('phmm_plan_create', 'phmm_plan_destroy', 'phmm_forward', 'phmm_estep',
           'phmm_estep_tables', 'phmm_estep_band', 'phmm_workspace_bytes', 'phmm_forward_ws', 'phmm_estep_ws',
           'phmm_estep_static', 'phmm_set_timing', 'phmm_kernel_times', 'phmm_kernel_time',
           'phmm_set_variant', 'phmm_set_spin_limit', 'phmm_set_tuning', 'phmm_get_tuning',
           'phmm_last_variant', 'phmm_last_launch_count',
           'phmm_last_error', 'phmm_version', 'phmm_mixdom2_class_subs_count', 'phmm_mixdom2_tables',
           'phmm_mixdom2_class_counts', 'phmm_tkf92_tables', 'phmm_mixdom2_chi',
           'phmm_mixdom2_chi_vjp_dirs', 'phmm_mixdom2_chi_vjp', 'phmm_fb1d_workspace_bytes', 'phmm_fb1d',
           'phmm_fb1d_emissions', 'phmm_viterbi_workspace_bytes', 'phmm_viterbi', 'phmm_holmes_rubin',
           'phmm_sample_workspace_bytes', 'phmm_sample_paths', 'phmm_pairs_count', 'phmm_pairs_decode',
           'phmm_estep_ws_prepare', 'phmm_estep_ws_launch', 'phmm_mixdom2_param_block_bytes',
           'phmm_mixdom2_param_block', 'phmm_mixdom2_tables_dp', 'phmm_mixdom2_class_counts_dp',
           'phmm_holmes_rubin_block_bytes', 'phmm_holmes_rubin_block', 'phmm_holmes_rubin_dp',
           'phmm_mixdom2_nest', 'phmm_mixdom2_nest_dp', 'phmm_nest_supported', 'phmm_mixdom2_tables_nest',
           'phmm_mixdom2_tables_nest_dp')


class Tuning(ctypes.Structure):
    """phmm_tuning: the launch configuration the autotuner searches."""
    _fields_ = [('variant', ctypes.c_int32), ('wave_per_sm', ctypes.c_int32),
                ('count_per_sm', ctypes.c_int32), ('priorities', ctypes.c_int32), ('checkpoint', ctypes.c_int32),
                ('tensor', ctypes.c_int32)]


class ModelDesc(ctypes.Structure):
    _fields_ = [('n_states', ctypes.c_int32),
                ('state_types', ctypes.POINTER(ctypes.c_int8)),
                ('state_group', ctypes.POINTER(ctypes.c_int32)),
                ('n_groups', ctypes.c_int32)]


class Batch(ctypes.Structure):
    _fields_ = [('n_pairs', ctypes.c_int32),
                ('Lx_host', ctypes.POINTER(ctypes.c_int32)),
                ('Ly_host', ctypes.POINTER(ctypes.c_int32)),
                ('residues', ctypes.c_void_p),
                ('x_off_host', ctypes.POINTER(ctypes.c_int64)),
                ('y_off_host', ctypes.POINTER(ctypes.c_int64)),
                ('chi', ctypes.c_void_p),
                ('chi_per_pair', ctypes.c_int32),
                ('emit_M', ctypes.c_void_p),
                ('emit_I', ctypes.c_void_p),
                ('emit_D', ctypes.c_void_p),
                ('emit_per_pair', ctypes.c_int32),
                ('cell_mask', ctypes.c_void_p),
                ('beam_log_width', ctypes.c_double),
                ('nest', ctypes.c_void_p),
                ('nest_dom', ctypes.c_int32),
                ('nest_frag', ctypes.c_int32)]


class MixDom2Params(ctypes.Structure):
    _fields_ = [('n_dom', ctypes.c_int32), ('n_frag', ctypes.c_int32),
                ('n_classes', ctypes.c_int32), ('alphabet', ctypes.c_int32),
                ('main_ins', ctypes.c_double), ('main_del', ctypes.c_double)] + [
        (name, ctypes.POINTER(ctypes.c_double)) for name in (
            'dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates', 'class_pis',
            'class_S_exch', 'classdist')]


class Tkf92Params(ctypes.Structure):
    _fields_ = [('ins_rate', ctypes.c_double), ('del_rate', ctypes.c_double), ('ext', ctypes.c_double),
                ('alphabet', ctypes.c_int32), ('Q', ctypes.POINTER(ctypes.c_double)),
                ('pi', ctypes.POINTER(ctypes.c_double))]


class Fb1dBatch(ctypes.Structure):
    _fields_ = [('n_pairs', ctypes.c_int32), ('n_states', ctypes.c_int32),
                ('L_host', ctypes.POINTER(ctypes.c_int32)), ('off_host', ctypes.POINTER(ctypes.c_int64)),
                ('emit', ctypes.c_void_p), ('chi', ctypes.c_void_p), ('chi_per_pair', ctypes.c_int32),
                ('init_state', ctypes.c_int32), ('final_state', ctypes.c_int32)]


class PairHMMError(RuntimeError):
    pass


def load(path=None):
    """Load libpairhmm.so (built in-tree by pairhmm.build / __graft_entry__.build)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise PairHMMError(f'CUDA library not built: {path} is missing '
                           '(run `python -c "import __graft_entry__ as g; g.build()"`)')
    lib = ctypes.CDLL(path)
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    lib.phmm_plan_create.argtypes = [ctypes.POINTER(ModelDesc), ctypes.POINTER(vp)]
    lib.phmm_plan_create.restype = ctypes.c_int
    lib.phmm_plan_destroy.argtypes = [vp]
    lib.phmm_plan_destroy.restype = None
    lib.phmm_forward.argtypes = [vp, ctypes.POINTER(Batch), vp, vp, vp]
    lib.phmm_forward.restype = ctypes.c_int
    lib.phmm_estep.argtypes = [vp, ctypes.POINTER(Batch), vp, vp, vp, vp, vp, vp, vp]
    lib.phmm_estep.restype = ctypes.c_int
    lib.phmm_estep_static.argtypes = [ctypes.POINTER(ModelDesc), ctypes.POINTER(Batch)] + [vp] * 7
    lib.phmm_estep_static.restype = ctypes.c_int
    lib.phmm_estep_tables.argtypes = [vp, ctypes.POINTER(Batch)] + [vp] * 10
    lib.phmm_estep_tables.restype = ctypes.c_int
    lib.phmm_estep_band.argtypes = [vp, ctypes.POINTER(Batch), vp, i32] + [vp] * 8
    lib.phmm_estep_band.restype = ctypes.c_int
    lib.phmm_workspace_bytes.argtypes = [vp, ctypes.POINTER(Batch), ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
    lib.phmm_workspace_bytes.restype = ctypes.c_int
    lib.phmm_forward_ws.argtypes = [vp, ctypes.POINTER(Batch), vp, ctypes.c_size_t, vp, vp, vp]
    lib.phmm_forward_ws.restype = ctypes.c_int
    lib.phmm_estep_ws.argtypes = [vp, ctypes.POINTER(Batch), vp, ctypes.c_size_t] + [vp] * 7
    lib.phmm_estep_ws.restype = ctypes.c_int
    lib.phmm_set_timing.argtypes = [vp, ctypes.c_int]
    lib.phmm_set_timing.restype = ctypes.c_int
    lib.phmm_kernel_times.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    lib.phmm_kernel_times.restype = ctypes.c_int
    lib.phmm_kernel_time.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
    lib.phmm_kernel_time.restype = ctypes.c_int
    lib.phmm_set_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    lib.phmm_set_tuning.restype = ctypes.c_int
    lib.phmm_get_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    lib.phmm_get_tuning.restype = ctypes.c_int
    lib.phmm_set_spin_limit.argtypes = [vp, ctypes.c_longlong]
    lib.phmm_set_spin_limit.restype = ctypes.c_int
    lib.phmm_set_variant.argtypes = [vp, ctypes.c_int]
    lib.phmm_set_variant.restype = ctypes.c_int
    lib.phmm_last_variant.argtypes = [vp]
    lib.phmm_last_variant.restype = ctypes.c_int
    lib.phmm_last_launch_count.argtypes = [vp]
    lib.phmm_last_launch_count.restype = ctypes.c_int
    lib.phmm_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.phmm_last_error.restype = ctypes.c_int
    lib.phmm_mixdom2_class_subs_count.argtypes = [ctypes.POINTER(MixDom2Params), ctypes.c_int32]
    lib.phmm_mixdom2_class_subs_count.restype = ctypes.c_size_t
    lib.phmm_mixdom2_tables.argtypes = [ctypes.POINTER(MixDom2Params), ctypes.c_int32] + [vp] * 7
    lib.phmm_mixdom2_tables.restype = ctypes.c_int
    lib.phmm_mixdom2_class_counts.argtypes = [ctypes.POINTER(MixDom2Params), ctypes.c_int32] + [vp] * 9
    lib.phmm_mixdom2_class_counts.restype = ctypes.c_int
    lib.phmm_mixdom2_chi.argtypes = [ctypes.POINTER(MixDom2Params), ctypes.c_int32] + [vp] * 4
    lib.phmm_mixdom2_chi.restype = ctypes.c_int
    lib.phmm_mixdom2_chi_vjp_dirs.argtypes = [ctypes.POINTER(MixDom2Params)]
    lib.phmm_mixdom2_chi_vjp_dirs.restype = ctypes.c_int
    lib.phmm_mixdom2_chi_vjp.argtypes = [ctypes.POINTER(MixDom2Params), ctypes.c_int32] + [vp] * 4
    lib.phmm_mixdom2_chi_vjp.restype = ctypes.c_int
    lib.phmm_tkf92_tables.argtypes = [ctypes.POINTER(Tkf92Params), ctypes.c_int32] + [vp] * 7
    lib.phmm_tkf92_tables.restype = ctypes.c_int
    lib.phmm_fb1d_workspace_bytes.argtypes = [ctypes.POINTER(Fb1dBatch), ctypes.POINTER(ctypes.c_size_t)]
    lib.phmm_fb1d_workspace_bytes.restype = ctypes.c_int
    lib.phmm_fb1d.argtypes = [ctypes.POINTER(Fb1dBatch), vp, ctypes.c_size_t, vp, vp, vp, vp, vp]
    lib.phmm_fb1d.restype = ctypes.c_int
    lib.phmm_fb1d_emissions.argtypes = [ctypes.POINTER(ModelDesc), ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int64), vp, vp, vp, vp, vp, vp, ctypes.c_int32,
                                        vp, ctypes.c_size_t, vp, vp, vp]
    lib.phmm_fb1d_emissions.restype = ctypes.c_int
    lib.phmm_viterbi_workspace_bytes.argtypes = [ctypes.POINTER(ModelDesc), ctypes.POINTER(Batch),
                                                 ctypes.POINTER(ctypes.c_size_t)]
    lib.phmm_viterbi_workspace_bytes.restype = ctypes.c_int
    lib.phmm_viterbi.argtypes = [ctypes.POINTER(ModelDesc), ctypes.POINTER(Batch)] + [vp] * 4 + \
        [vp, ctypes.c_size_t, vp, vp, vp, vp, vp]
    lib.phmm_viterbi.restype = ctypes.c_int
    lib.phmm_sample_workspace_bytes.argtypes = [ctypes.POINTER(ModelDesc), ctypes.POINTER(Batch),
                                                ctypes.POINTER(ctypes.c_size_t)]
    lib.phmm_sample_workspace_bytes.restype = ctypes.c_int
    lib.phmm_sample_paths.argtypes = [ctypes.POINTER(ModelDesc), ctypes.POINTER(Batch)] + [vp] * 4 + \
        [ctypes.c_int32, ctypes.c_uint64, vp, ctypes.c_size_t, vp, vp, vp, vp, vp]
    lib.phmm_sample_paths.restype = ctypes.c_int
    lib.phmm_holmes_rubin.argtypes = [ctypes.c_int32, ctypes.c_int32, vp, vp, ctypes.c_int32, vp, vp, vp, vp, vp]
    lib.phmm_holmes_rubin.restype = ctypes.c_int
    lib.phmm_estep_ws_prepare.argtypes = [vp, ctypes.POINTER(Batch), vp, ctypes.c_size_t, vp]
    lib.phmm_estep_ws_prepare.restype = ctypes.c_int
    lib.phmm_estep_ws_launch.argtypes = [vp, ctypes.POINTER(Batch), vp, ctypes.c_size_t] + [vp] * 7
    lib.phmm_estep_ws_launch.restype = ctypes.c_int
    lib.phmm_mixdom2_param_block_bytes.argtypes = []
    lib.phmm_mixdom2_param_block_bytes.restype = ctypes.c_size_t
    lib.phmm_mixdom2_param_block.argtypes = [ctypes.POINTER(MixDom2Params), vp, ctypes.c_size_t]
    lib.phmm_mixdom2_param_block.restype = ctypes.c_int
    lib.phmm_mixdom2_tables_dp.argtypes = [vp] + [ctypes.c_int32] * 4 + [vp] * 7
    lib.phmm_mixdom2_tables_dp.restype = ctypes.c_int
    lib.phmm_mixdom2_nest.argtypes = [ctypes.POINTER(MixDom2Params), ctypes.c_int32, vp, vp, vp]
    lib.phmm_mixdom2_nest.restype = ctypes.c_int
    lib.phmm_mixdom2_nest_dp.argtypes = [vp] + [ctypes.c_int32] * 4 + [vp] * 3
    lib.phmm_mixdom2_nest_dp.restype = ctypes.c_int
    lib.phmm_mixdom2_tables_nest.argtypes = [ctypes.POINTER(MixDom2Params), ctypes.c_int32] + [vp] * 8
    lib.phmm_mixdom2_tables_nest.restype = ctypes.c_int
    lib.phmm_mixdom2_tables_nest_dp.argtypes = [vp] + [ctypes.c_int32] * 4 + [vp] * 8
    lib.phmm_mixdom2_tables_nest_dp.restype = ctypes.c_int
    lib.phmm_nest_supported.argtypes = [ctypes.c_int32, ctypes.c_int32]
    lib.phmm_nest_supported.restype = ctypes.c_int
    lib.phmm_mixdom2_class_counts_dp.argtypes = [vp] + [ctypes.c_int32] * 4 + [vp] * 9
    lib.phmm_mixdom2_class_counts_dp.restype = ctypes.c_int
    lib.phmm_holmes_rubin_block_bytes.argtypes = [ctypes.c_int32]
    lib.phmm_holmes_rubin_block_bytes.restype = ctypes.c_size_t
    lib.phmm_holmes_rubin_block.argtypes = [ctypes.c_int32, ctypes.c_int32, vp, vp, vp, ctypes.c_size_t]
    lib.phmm_holmes_rubin_block.restype = ctypes.c_int
    lib.phmm_holmes_rubin_dp.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, vp, vp, vp, vp, vp]
    lib.phmm_holmes_rubin_dp.restype = ctypes.c_int
    lib.phmm_version.argtypes = []
    lib.phmm_version.restype = ctypes.c_int
    _LIB = lib
    return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(1024)
    lib.phmm_last_error(buf, 1024)
    return buf.value.decode()


def _check(rc, what):
    if rc != 0:
        raise PairHMMError(f'{what} failed ({rc}): {last_error()}')


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class Plan:
    """A plan for one pair-HMM state space (phmm_plan_create)."""

    def __init__(self, state_types, state_groups, n_groups):
        self.lib = load()
        st = np.ascontiguousarray(np.asarray(state_types, dtype=np.int8))
        gr = np.ascontiguousarray(np.asarray(state_groups, dtype=np.int32))
        self.n_states = int(st.size)
        self.n_groups = int(n_groups)
        self._st, self._gr = st, gr
        desc = ModelDesc(self.n_states, st.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)),
                         gr.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), self.n_groups)
        h = ctypes.c_void_p()
        _check(self.lib.phmm_plan_create(ctypes.byref(desc), ctypes.byref(h)), 'phmm_plan_create')
        self.handle = h

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h is not None and h.value:
            try:
                self.lib.phmm_plan_destroy(h)
            except Exception:
                pass
            self.handle = None

    @property
    def launches(self):
        return self.lib.phmm_last_launch_count(self.handle)

    def set_variant(self, variant):
        """0 automatic, 1 generic, 2 register-resident warp, 3 quad-per-warp block
        kernels, 4 split warp E-step (forward || backward recursion, then counts),
        5 split block E-step, 6 wide kernels, 7 split E-step on two-warp stripes."""
        _check(self.lib.phmm_set_variant(self.handle, int(variant)), 'phmm_set_variant')

    @property
    def last_variant(self):
        return self.lib.phmm_last_variant(self.handle)

    def set_timing(self, enable=True):
        _check(self.lib.phmm_set_timing(self.handle, int(enable)), 'phmm_set_timing')

    def set_tuning(self, variant=0, wave_per_sm=0, count_per_sm=-1, priorities=0, checkpoint=0, tensor=0):
        """Launch configuration (phmm_set_tuning): kernel family, resident CTAs
        per SM of each wavefront grid (0 automatic), of the overlapped count
        grid (-1 automatic, 0 none), wavefront/count stream priorities,
        stripe-edge checkpointing of the wide kernels' E-step (0 automatic,
        1 on, 2 off), and the wide forward contraction on the tensor cores as
        3xTF32 (tensor=1)."""
        t = Tuning(int(variant), int(wave_per_sm), int(count_per_sm), int(priorities), int(checkpoint),
                   int(tensor))
        _check(self.lib.phmm_set_tuning(self.handle, ctypes.byref(t)), 'phmm_set_tuning')

    def get_tuning(self):
        t = Tuning()
        _check(self.lib.phmm_get_tuning(self.handle, ctypes.byref(t)), 'phmm_get_tuning')
        return {'variant': t.variant, 'wave_per_sm': t.wave_per_sm, 'count_per_sm': t.count_per_sm,
                'priorities': t.priorities, 'checkpoint': t.checkpoint, 'tensor': t.tensor}

    def set_spin_limit(self, iterations=0):
        """Bound of the kernels' inter-CTA waits in polling iterations (0: the
        default, about 5 s); a wait that reaches it marks its pair
        PHMM_ST_TIMEOUT with a NEG_INF log-likelihood (phmm_set_spin_limit)."""
        _check(self.lib.phmm_set_spin_limit(self.handle, int(iterations)), 'phmm_set_spin_limit')

    def kernel_time(self, which):
        """Device ms of kernel `which` (0 forward, 1 backward, 2 split count pass)
        of the last timed call."""
        a = ctypes.c_float()
        _check(self.lib.phmm_kernel_time(self.handle, int(which), ctypes.byref(a)), 'phmm_kernel_time')
        return float(a.value)

    def kernel_times(self):
        """(forward_ms, backward_ms) of the last call (CUDA events on its stream)."""
        a, b = ctypes.c_float(), ctypes.c_float()
        _check(self.lib.phmm_kernel_times(self.handle, ctypes.byref(a), ctypes.byref(b)),
               'phmm_kernel_times')
        return float(a.value), float(b.value)


@dataclass
class DeviceBatch:
    """Device-resident inputs of one batch plus the host length arrays."""
    Lx: np.ndarray
    Ly: np.ndarray
    x_off: np.ndarray
    y_off: np.ndarray
    residues: torch.Tensor      # uint8 [total]
    chi: torch.Tensor           # float32 [P or 1, N, N]
    emit_M: torch.Tensor        # float32 [P or 1, G, 21, 21]
    emit_I: torch.Tensor        # float32 [P or 1, G, 21]
    emit_D: torch.Tensor        # float32 [P or 1, G, 21]
    cell_mask: torch.Tensor = None   # uint8 [sum (Lx+1)(Ly+1)]: bit 0 M, 1 I, 2 D may emit
    beam_log_width: float = 0.0      # > 0: beam pruning of the forward (generic kernels)
    nest: torch.Tensor = None        # float32 [P or 1, R]: factored MixDom transitions (models.nested_record)
    nest_kf: tuple = (0, 0)          # (K, F) of the nest records
    _struct: Batch = field(default=None, repr=False)

    @property
    def n_pairs(self):
        return int(self.Lx.size)

    def struct(self):
        if self._struct is None:
            P = self.n_pairs
            self._struct = Batch(
                P,
                self.Lx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                self.Ly.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                ctypes.c_void_p(self.residues.data_ptr()),
                self.x_off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                self.y_off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                ctypes.c_void_p(self.chi.data_ptr()),
                int(self.chi.shape[0] == P),
                ctypes.c_void_p(self.emit_M.data_ptr()),
                ctypes.c_void_p(self.emit_I.data_ptr()),
                ctypes.c_void_p(self.emit_D.data_ptr()),
                int(self.emit_M.shape[0] == P),
                ctypes.c_void_p(self.cell_mask.data_ptr() if self.cell_mask is not None else 0),
                float(self.beam_log_width),
                ctypes.c_void_p(self.nest.data_ptr() if self.nest is not None else 0),
                int(self.nest_kf[0]) if self.nest is not None else 0,
                int(self.nest_kf[1]) if self.nest is not None else 0)
        return self._struct


def pack_residues(xs, ys):
    """Concatenate residues of all pairs: [x_0, y_0, x_1, y_1, ...] (uint8)."""
    P = len(xs)
    if len(ys) != P:
        raise ValueError('xs and ys must hold the same number of sequences')
    parts = [None] * (2 * P)
    parts[0::2] = xs
    parts[1::2] = ys
    lens = np.fromiter(map(len, parts), dtype=np.int64, count=2 * P)
    offs = np.zeros(2 * P, np.int64)
    if P:
        np.cumsum(lens[:-1], out=offs[1:])
    allr = np.concatenate(parts) if lens.sum() else np.zeros(0, np.int64)
    if allr.ndim != 1:
        raise ValueError('sequences must be one-dimensional')
    if allr.dtype.kind not in 'iu':
        allr = allr.astype(np.int64)
    if allr.size and (allr.min() < 0 or allr.max() > 20):
        raise ValueError('residues must be integers in 0..20 (20 = wildcard)')
    buf = allr.astype(np.uint8)
    if buf.size == 0:
        buf = np.zeros(16, np.uint8)
    return (buf, offs[0::2].copy(), offs[1::2].copy(),
            lens[0::2].astype(np.int32), lens[1::2].astype(np.int32))


def to_host(tensors):
    """Copy a dict of device tensors to host numpy arrays with one
    synchronisation.  The arrays are views of one pinned block from torch's
    caching host allocator (no host-side copy; the block returns to the cache
    when the arrays are dropped).  Tensors that are contiguous views of one
    device buffer (the batched E-steps' output arena) come back in a single
    copy of that buffer; others are copied one by one into the block."""
    items = [(k, v) for k, v in tensors.items() if isinstance(v, torch.Tensor)]
    if not items:
        return dict(tensors)
    dev = items[0][1].device
    if dev.type != 'cuda':
        return {k: (v.numpy() if isinstance(v, torch.Tensor) else v) for k, v in tensors.items()}
    stream = torch.cuda.current_stream(dev)
    stor = items[0][1].untyped_storage()
    base, nb = stor.data_ptr(), stor.nbytes()
    # one device buffer holds them all (an output arena): its bytes come back in
    # one copy and the arrays are numpy views of the pinned block
    shared = all(v.device == dev and v.dtype in _NP_DTYPE and v.is_contiguous()
                 and base <= v.data_ptr() and v.data_ptr() + v.numel() * v.element_size() <= base + nb
                 for _, v in items)
    views = {}
    if shared:
        host = torch.empty(nb, dtype=torch.uint8, pin_memory=True)
        src = torch.empty(0, dtype=torch.uint8, device=dev).set_(stor, 0, (nb,))
        host.copy_(src, non_blocking=True)
        hn = host.numpy()
        for k, v in items:
            o = v.data_ptr() - base
            views[k] = hn[o:o + v.numel() * v.element_size()].view(_NP_DTYPE[v.dtype]).reshape(v.shape)
        stream.synchronize()
        out = dict(tensors)
        out.update(views)
        return out
    sizes = [(v.numel() * v.element_size() + 255) // 256 * 256 for _, v in items]
    host = torch.empty(max(sum(sizes), 1), dtype=torch.uint8, pin_memory=True)
    o = 0
    for (k, v), n in zip(items, sizes):
        hv = host[o:o + v.numel() * v.element_size()].view(v.dtype).view(v.shape)
        hv.copy_(v if v.is_contiguous() else v.contiguous(), non_blocking=True)
        views[k] = hv
        o += n
    stream.synchronize()
    out = {k: v.numpy() for k, v in views.items()}
    for k, v in tensors.items():
        if k not in out:
            out[k] = v
    return out


_ESIZE = {torch.float64: 8, torch.float32: 4, torch.int64: 8, torch.int32: 4, torch.uint8: 1}
_NP_DTYPE = {torch.float64: np.float64, torch.float32: np.float32, torch.int64: np.int64, torch.int32: np.int32,
             torch.uint8: np.uint8}


def arena_layout(specs):
    """Layout of an output arena: specs is a list of (name, shape, dtype), each
    slice 256-byte aligned.  Returns ([(name, dtype, shape, strides, element
    offset)], bytes)."""
    lay, o = [], 0
    for name, shape, dt in specs:
        shape = tuple(int(s) for s in shape)
        esz = _ESIZE[dt]
        st, n = [], 1
        for s in reversed(shape):
            st.append(n)
            n *= s
        lay.append((name, dt, shape, tuple(reversed(st)), o // esz))
        o += (n * esz + 255) // 256 * 256
    return lay, max(o, 256)


def arena_views(buf, layout):
    """The named tensors of an arena layout over the uint8 buffer buf (one
    strided view each: a call returning many outputs pays one view per output)."""
    typed, out = {}, {}
    for name, dt, shape, st, off in layout:
        v = typed.get(dt)
        if v is None:
            v = typed[dt] = buf.view(dt)
        out[name] = v.as_strided(shape, st, off)
    return out


class OutputArena:
    """One device buffer carved into the output tensors of a call, so that
    to_host brings them back in a single copy."""

    def __init__(self, device, specs):
        # specs: list of (name, shape, dtype); each slice 256-byte aligned
        self.layout, nb = arena_layout(specs)
        self.buf = torch.empty(nb, dtype=torch.uint8, device=device)
        self.t = arena_views(self.buf, self.layout)

    def __getitem__(self, name):
        return self.t[name]


def make_batch(xs, ys, chi, emit_M, emit_I, emit_D, device='cuda', cell_masks=None, beam_log_width=0.0,
               nest=None, nest_kf=None):
    """Build a DeviceBatch from host sequences and float tables.

    chi: [P or 1, N, N]; emit_*: [P or 1, G, ...] (numpy or torch, any float);
    cell_masks: optional list of per-pair uint8 arrays (Lx+1, Ly+1) (bit 0 M,
    1 I, 2 D may emit at the cell); nest: optional [P or 1, R] factored
    MixDom transitions of chi (models.nested_record) with nest_kf = (K, F)."""
    buf, xo, yo, Lx, Ly = pack_residues(xs, ys)

    def dev(a, dt):
        t = torch.as_tensor(np.asarray(a) if not isinstance(a, torch.Tensor) else a)
        return t.to(device=device, dtype=dt).contiguous()
    cm = None
    if cell_masks is not None:
        if len(cell_masks) != Lx.size:
            raise ValueError('one cell mask per pair')
        for m, a, b in zip(cell_masks, Lx, Ly):
            if tuple(np.shape(m)) != (int(a) + 1, int(b) + 1):
                raise ValueError('cell mask of a pair must have shape (Lx+1, Ly+1)')
        flat = np.concatenate([np.asarray(m, np.uint8).reshape(-1) for m in cell_masks]) if len(cell_masks) \
            else np.zeros(1, np.uint8)
        cm = dev(flat, torch.uint8)
    return DeviceBatch(Lx=Lx, Ly=Ly, x_off=xo, y_off=yo,
                       residues=dev(buf, torch.uint8), chi=dev(chi, torch.float32),
                       emit_M=dev(emit_M, torch.float32), emit_I=dev(emit_I, torch.float32),
                       emit_D=dev(emit_D, torch.float32), cell_mask=cm,
                       beam_log_width=float(beam_log_width),
                       nest=None if nest is None else dev(nest, torch.float32),
                       nest_kf=(0, 0) if nest is None else tuple(int(v) for v in nest_kf))


def forward(plan, batch, stream=None):
    """phmm_forward -> (ll float64 [P] tensor, status int32 [P] tensor) on the device."""
    P = batch.n_pairs
    dev = batch.residues.device
    ll = torch.empty(P, dtype=torch.float64, device=dev)
    st = torch.empty(P, dtype=torch.int32, device=dev)
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _check(plan.lib.phmm_forward(plan.handle, ctypes.byref(batch.struct()), _ptr(ll), _ptr(st),
                                 ctypes.c_void_p(s.cuda_stream)), 'phmm_forward')
    return ll, st


def estep(plan, batch, stream=None, out=None):
    """phmm_estep -> dict of device tensors (ll, n_trans, cnt_M, cnt_I, cnt_D, status)."""
    P = batch.n_pairs
    N, G = plan.n_states, plan.n_groups
    dev = batch.residues.device
    if out is None:
        out = {
            'll': torch.empty(P, dtype=torch.float64, device=dev),
            'n_trans': torch.empty(P, N, N, dtype=torch.float64, device=dev),
            'cnt_M': torch.empty(P, G, 21, 21, dtype=torch.float64, device=dev),
            'cnt_I': torch.empty(P, G, 21, dtype=torch.float64, device=dev),
            'cnt_D': torch.empty(P, G, 21, dtype=torch.float64, device=dev),
            'status': torch.empty(P, dtype=torch.int32, device=dev),
        }
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _check(plan.lib.phmm_estep(plan.handle, ctypes.byref(batch.struct()), _ptr(out['ll']),
                               _ptr(out['n_trans']), _ptr(out['cnt_M']), _ptr(out['cnt_I']),
                               _ptr(out['cnt_D']), _ptr(out['status']),
                               ctypes.c_void_p(s.cuda_stream)), 'phmm_estep')
    return out


def workspace_bytes(plan, batch, estep=True):
    """phmm_workspace_bytes: device scratch one *_ws call on `batch` needs.

    `batch` is a DeviceBatch or anything with a ``struct()`` giving the C
    struct; only its host length and offset arrays are read."""
    n = ctypes.c_size_t()
    _check(plan.lib.phmm_workspace_bytes(plan.handle, ctypes.byref(batch.struct()), int(bool(estep)),
                                         ctypes.byref(n)), 'phmm_workspace_bytes')
    return int(n.value)


def host_batch(Lx, Ly):
    """A length-only batch descriptor (no device data) for workspace queries."""
    Lx = np.ascontiguousarray(Lx, dtype=np.int32)
    Ly = np.ascontiguousarray(Ly, dtype=np.int32)
    xo = np.zeros(Lx.size, np.int64)
    yo = np.zeros(Lx.size, np.int64)
    z = torch.zeros(0)
    return DeviceBatch(Lx=Lx, Ly=Ly, x_off=xo, y_off=yo, residues=z, chi=z, emit_M=z, emit_I=z, emit_D=z)


def estep_ws(plan, batch, workspace, stream=None, out=None):
    """phmm_estep_ws: phmm_estep with scratch carved from `workspace` (a uint8
    device tensor or a (pointer, bytes) pair); allocates nothing."""
    P = batch.n_pairs
    N, G = plan.n_states, plan.n_groups
    dev = batch.residues.device
    if out is None:
        out = {
            'll': torch.empty(P, dtype=torch.float64, device=dev),
            'n_trans': torch.empty(P, N, N, dtype=torch.float64, device=dev),
            'cnt_M': torch.empty(P, G, 21, 21, dtype=torch.float64, device=dev),
            'cnt_I': torch.empty(P, G, 21, dtype=torch.float64, device=dev),
            'cnt_D': torch.empty(P, G, 21, dtype=torch.float64, device=dev),
            'status': torch.empty(P, dtype=torch.int32, device=dev),
        }
    if isinstance(workspace, torch.Tensor):
        wptr, wbytes = workspace.data_ptr(), workspace.numel() * workspace.element_size()
    else:
        wptr, wbytes = workspace
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _check(plan.lib.phmm_estep_ws(plan.handle, ctypes.byref(batch.struct()), ctypes.c_void_p(wptr),
                                  ctypes.c_size_t(wbytes), _ptr(out['ll']), _ptr(out['n_trans']),
                                  _ptr(out['cnt_M']), _ptr(out['cnt_I']), _ptr(out['cnt_D']),
                                  _ptr(out['status']), ctypes.c_void_p(s.cuda_stream)), 'phmm_estep_ws')
    return out


def estep_tables(plan, batch, want_F=True, want_B=True, want_post=True, stream=None):
    """phmm_estep_tables: E-step plus full lattice tables (API-parity path)."""
    P = batch.n_pairs
    N = plan.n_states
    dev = batch.residues.device
    cells = int(((batch.Lx.astype(np.int64) + 1) * (batch.Ly.astype(np.int64) + 1)).sum())
    G = plan.n_groups
    out = {
        'll': torch.empty(P, dtype=torch.float64, device=dev),
        'n_trans': torch.empty(P, N, N, dtype=torch.float64, device=dev),
        'cnt_M': torch.empty(P, G, 21, 21, dtype=torch.float64, device=dev),
        'cnt_I': torch.empty(P, G, 21, dtype=torch.float64, device=dev),
        'cnt_D': torch.empty(P, G, 21, dtype=torch.float64, device=dev),
        'status': torch.empty(P, dtype=torch.int32, device=dev),
        'log_F': torch.empty(cells, N, dtype=torch.float64, device=dev) if want_F else None,
        'log_B': torch.empty(cells, N, dtype=torch.float64, device=dev) if want_B else None,
        'post': torch.empty(cells, N, dtype=torch.float64, device=dev) if want_post else None,
    }
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _check(plan.lib.phmm_estep_tables(
        plan.handle, ctypes.byref(batch.struct()), _ptr(out['ll']), _ptr(out['n_trans']),
        _ptr(out['cnt_M']), _ptr(out['cnt_I']), _ptr(out['cnt_D']), _ptr(out['status']),
        _ptr(out['log_F']), _ptr(out['log_B']), _ptr(out['post']),
        ctypes.c_void_p(s.cuda_stream)), 'phmm_estep_tables')
    return out


def estep_band(plan, batch, band_centers, band_half_width, stream=None):
    """phmm_estep_band: E-step of a banded batch (its cell masks hold the
    bands) with posteriors in band layout.  band_centers: per pair an int
    array of Lx+1 centre columns.  Returns the phmm_estep outputs plus
    'post_band' [sum(Lx+1), 2W+1, N] float64 (pairs' rows concatenated)."""
    P = batch.n_pairs
    N = plan.n_states
    G = plan.n_groups
    dev = batch.residues.device
    W = int(band_half_width)
    centers = np.concatenate([np.asarray(c, np.int32)[:int(a) + 1] for c, a in zip(band_centers, batch.Lx)])
    if centers.size != int((batch.Lx.astype(np.int64) + 1).sum()):
        raise ValueError('band_centers: Lx+1 centre columns per pair')
    d_centers = torch.as_tensor(centers).to(dev)
    out = {
        'll': torch.empty(P, dtype=torch.float64, device=dev),
        'n_trans': torch.empty(P, N, N, dtype=torch.float64, device=dev),
        'cnt_M': torch.empty(P, G, 21, 21, dtype=torch.float64, device=dev),
        'cnt_I': torch.empty(P, G, 21, dtype=torch.float64, device=dev),
        'cnt_D': torch.empty(P, G, 21, dtype=torch.float64, device=dev),
        'status': torch.empty(P, dtype=torch.int32, device=dev),
        'post_band': torch.empty(centers.size, 2 * W + 1, N, dtype=torch.float64, device=dev),
    }
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _check(plan.lib.phmm_estep_band(
        plan.handle, ctypes.byref(batch.struct()), _ptr(d_centers), W, _ptr(out['ll']), _ptr(out['n_trans']),
        _ptr(out['cnt_M']), _ptr(out['cnt_I']), _ptr(out['cnt_D']), _ptr(out['status']), _ptr(out['post_band']),
        ctypes.c_void_p(s.cuda_stream)), 'phmm_estep_band')
    out['_centers'] = d_centers   # kept alive until the stream has read it
    return out


class MixDom2Prologue:
    """phmm_mixdom2_tables for one MixDom2 parameter set: packs the host
    parameter arrays once, then builds the E-step inputs of any batch of
    per-pair times on the device.

    params: the MixDom2 parameter dict (main_ins, main_del, dom_ins, dom_del,
    dom_weights, frag_weights, ext_rates [K,F] or [K,F,F], class_pis,
    class_S_exch, classdist)."""

    KEYS = ('dom_ins', 'dom_del', 'dom_weights', 'frag_weights', 'ext_rates', 'class_pis',
            'class_S_exch', 'classdist')

    def __init__(self, params):
        self.lib = load()
        host = lambda v: v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else v
        arr = {k: np.ascontiguousarray(np.asarray(host(params[k]), dtype=np.float64)) for k in self.KEYS}
        self.K = arr['dom_ins'].size
        self.F = arr['frag_weights'].shape[-1]
        self.C, self.A = arr['class_pis'].shape
        if arr['ext_rates'].ndim == 2:
            arr['ext_rates'] = np.ascontiguousarray(np.einsum('kf,fg->kfg', arr['ext_rates'], np.eye(self.F)))
        self._arr = arr   # the struct points into these arrays
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self.struct = MixDom2Params(self.K, self.F, self.C, self.A, float(host(params['main_ins'])),
                                    float(host(params['main_del'])), *[dp(arr[k]) for k in self.KEYS])
        self.N, self.G = 2 + 5 * self.K * self.F, self.K * self.F

    def class_Q(self):
        """The class rate matrices Q_c[a,b] = S_c[a,b] pi_c[b] with rows summing
        to zero (train/vjp.py:463-476), float64 [C,A,A] on the host."""
        if getattr(self, '_Q', None) is None:
            Q = self._arr['class_S_exch'] * self._arr['class_pis'][:, None, :]
            for c in range(Q.shape[0]):
                np.fill_diagonal(Q[c], 0.0)
                np.fill_diagonal(Q[c], -Q[c].sum(axis=1))
            self._Q = np.ascontiguousarray(Q)
        return self._Q

    def shapes(self, P):
        """(chi, emit_M, emit_I, emit_D, class_subs) shapes for P pairs."""
        N, G = self.N, self.G
        return (P, N, N), (P, G, 21, 21), (P, G, 21), (P, G, 21), (P, self.C, self.A, self.A)

    def run(self, t, chi, EM, EI, ED, csubs, stream=None, nest=None):
        """Write into caller tensors: t float64 [P] and the five outputs of
        shapes(P) (and the factored record into `nest`, when given)."""
        P = t.numel()
        s = stream if stream is not None else torch.cuda.current_stream(t.device)
        if nest is not None:
            _check(self.lib.phmm_mixdom2_tables_nest(ctypes.byref(self.struct), P, _ptr(t), _ptr(chi), _ptr(EM),
                                                     _ptr(EI), _ptr(ED), _ptr(csubs), _ptr(nest),
                                                     ctypes.c_void_p(s.cuda_stream)), 'phmm_mixdom2_tables_nest')
            return
        _check(self.lib.phmm_mixdom2_tables(ctypes.byref(self.struct), P, _ptr(t), _ptr(chi), _ptr(EM), _ptr(EI),
                                            _ptr(ED), _ptr(csubs), ctypes.c_void_p(s.cuda_stream)),
               'phmm_mixdom2_tables')

    def nest_supported(self):
        """True when the E-step kernels contract this layout (K, F) through the factored record."""
        return bool(self.lib.phmm_nest_supported(self.K, self.F))

    def nest(self, t, stream=None, out=None):
        """phmm_mixdom2_nest: the factored transitions (phmm_batch.nest), float32
        [P, 20KF + 25KF^2] on t's device, for float64 device times t [P]."""
        P = t.numel()
        R = 20 * self.K * self.F + 25 * self.K * self.F * self.F
        if out is None:
            out = torch.empty(P, R, dtype=torch.float32, device=t.device)
        s = stream if stream is not None else torch.cuda.current_stream(t.device)
        _check(self.lib.phmm_mixdom2_nest(ctypes.byref(self.struct), P, _ptr(t), _ptr(out),
                                          ctypes.c_void_p(s.cuda_stream)), 'phmm_mixdom2_nest')
        return out

    def class_count_shapes(self, P):
        C, A = self.C, self.A
        return {'class_match_counts': (P, C, A, A), 'class_insert_counts': (P, C, A),
                'class_delete_counts': (P, C, A), 'classdist_counts': (P, self.K, self.F, C)}

    def class_counts(self, csubs, cnt_M, cnt_I, cnt_D, stream=None, out=None):
        """phmm_mixdom2_class_counts: the per-class counts of e_step_mixdom2
        (class_match_counts [P,C,20,20], class_insert_counts / class_delete_counts
        [P,C,20], classdist_counts [P,K,F,C]) as float64 device tensors (written
        into `out` when given)."""
        P, dev, f64 = csubs.shape[0], csubs.device, torch.float64
        if out is None:
            out = {k: torch.empty(*sh, dtype=f64, device=dev) for k, sh in self.class_count_shapes(P).items()}
        s = stream if stream is not None else torch.cuda.current_stream(dev)
        _check(self.lib.phmm_mixdom2_class_counts(
            ctypes.byref(self.struct), P, _ptr(csubs), _ptr(cnt_M.contiguous()), _ptr(cnt_I.contiguous()),
            _ptr(cnt_D.contiguous()), *[_ptr(v) for v in out.values()], ctypes.c_void_p(s.cuda_stream)),
            'phmm_mixdom2_class_counts')
        return out

    def chi(self, t, stream=None):
        """phmm_mixdom2_chi: (chi float32, chi float64) [P,N,N] for float64 device times t [P]."""
        P = t.numel()
        c32 = torch.empty(P, self.N, self.N, dtype=torch.float32, device=t.device)
        c64 = torch.empty(P, self.N, self.N, dtype=torch.float64, device=t.device)
        s = stream if stream is not None else torch.cuda.current_stream(t.device)
        _check(self.lib.phmm_mixdom2_chi(ctypes.byref(self.struct), P, _ptr(t), _ptr(c32), _ptr(c64),
                                         ctypes.c_void_p(s.cuda_stream)), 'phmm_mixdom2_chi')
        return c32, c64

    def chi_vjp(self, t, grad_chi, stream=None):
        """phmm_mixdom2_chi_vjp: [P, n_dirs] float64 directional contractions
        (directions: main_ins, main_del, t, then dom_ins, dom_del, dom_weights,
        frag_weights, ext_rates [K,F,F] entries)."""
        P = t.numel()
        nd = self.lib.phmm_mixdom2_chi_vjp_dirs(ctypes.byref(self.struct))
        g = grad_chi.to(torch.float64).contiguous()
        out = torch.empty(P, nd, dtype=torch.float64, device=t.device)
        s = stream if stream is not None else torch.cuda.current_stream(t.device)
        _check(self.lib.phmm_mixdom2_chi_vjp(ctypes.byref(self.struct), P, _ptr(t), _ptr(g), _ptr(out),
                                             ctypes.c_void_p(s.cuda_stream)), 'phmm_mixdom2_chi_vjp')
        return out

    def __call__(self, ts, device='cuda', stream=None, with_nest=False):
        """(chi, EM, EI, ED, csubs) on the device for per-pair times ts; with
        with_nest, the factored record (phmm_batch.nest) appended, built by
        the same launch."""
        if isinstance(ts, torch.Tensor):
            t = ts.to(device=device, dtype=torch.float64).reshape(-1).contiguous()
        else:
            t = torch.from_numpy(np.ascontiguousarray(np.asarray(ts, np.float64).reshape(-1))).to(device)
        shp = self.shapes(t.numel())
        f32, f64 = torch.float32, torch.float64
        outs = [torch.empty(sh, dtype=f64 if i == 4 else f32, device=t.device) for i, sh in enumerate(shp)]
        nest = None
        if with_nest:
            R = 20 * self.K * self.F + 25 * self.K * self.F * self.F
            nest = torch.empty(t.numel(), R, dtype=f32, device=t.device)
        self.run(t, *outs, stream=stream, nest=nest)
        return tuple(outs) + ((nest,) if with_nest else ())


def mixdom2_tables(params, ts, device='cuda', stream=None):
    """The MixDom2 E-step inputs built on the device: (chi [P,N,N] f32,
    EM [P,G,21,21] f32, EI [P,G,21] f32, ED [P,G,21] f32, csubs [P,C,20,20]
    f64) for per-pair times ts."""
    return MixDom2Prologue(params)(ts, device=device, stream=stream)


class Tkf92Prologue:
    """phmm_tkf92_tables for one TKF92 parameter set (ext = 0: TKF91): packs
    the host parameters once, then builds the E-step inputs of any batch of
    per-pair times on the device."""

    def __init__(self, ins_rate, del_rate, ext, Q, pi):
        self.lib = load()
        host = lambda v: v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else v
        self._Q = np.ascontiguousarray(np.asarray(host(Q), dtype=np.float64))
        self._pi = np.ascontiguousarray(np.asarray(host(pi), dtype=np.float64).reshape(-1))
        self.A = self._pi.size
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self.struct = Tkf92Params(float(host(ins_rate)), float(host(del_rate)), float(host(ext)), self.A,
                                  dp(self._Q), dp(self._pi))

    def shapes(self, P):
        """(chi, emit_M, emit_I, emit_D, sub) shapes for P pairs."""
        return (P, 5, 5), (P, 1, 21, 21), (P, 1, 21), (P, 1, 21), (P, self.A, self.A)

    def run(self, t, chi, EM, EI, ED, sub, stream=None):
        """Write into caller tensors: t float64 [P] and the five outputs of shapes(P)."""
        P = t.numel()
        s = stream if stream is not None else torch.cuda.current_stream(t.device)
        _check(self.lib.phmm_tkf92_tables(ctypes.byref(self.struct), P, _ptr(t), _ptr(chi), _ptr(EM), _ptr(EI),
                                          _ptr(ED), _ptr(sub), ctypes.c_void_p(s.cuda_stream)), 'phmm_tkf92_tables')

    def __call__(self, ts, device='cuda', stream=None):
        if isinstance(ts, torch.Tensor):
            t = ts.to(device=device, dtype=torch.float64).reshape(-1).contiguous()
        else:
            t = torch.from_numpy(np.ascontiguousarray(np.asarray(ts, np.float64).reshape(-1))).to(device)
        shp = self.shapes(t.numel())
        outs = [torch.empty(sh, dtype=torch.float64 if i == 4 else torch.float32, device=t.device)
                for i, sh in enumerate(shp)]
        self.run(t, *outs, stream=stream)
        return tuple(outs)


def tkf92_tables(ins_rate, del_rate, ext, Q, pi, ts, device='cuda', stream=None):
    """The TKF92 (ext = 0: TKF91) E-step inputs built on the device for per-pair
    times ts: (chi [P,5,5] f32, EM [P,1,21,21] f32, EI [P,1,21] f32, ED
    [P,1,21] f32, sub [P,20,20] f64) device tensors."""
    return Tkf92Prologue(ins_rate, del_rate, ext, Q, pi)(ts, device=device, stream=stream)


def sample_paths(state_types, groups, G, xs, ys, log_chi, log_M, log_I, log_D, n_samples, seed,
                 device='cuda', stream=None):
    """phmm_sample_paths: (ll [P] float64 numpy, paths: per pair a list of
    n_samples [n, 3] int32 arrays of (i, j, state)).  Inputs as viterbi()."""
    lib = load()
    st_arr = np.ascontiguousarray(np.asarray(state_types, np.int8))
    gr = np.ascontiguousarray(np.asarray(groups, np.int32))
    md = ModelDesc(st_arr.size, st_arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)),
                   gr.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), int(G))
    buf, xo, yo, Lx, Ly = pack_residues(xs, ys)
    P, S = Lx.size, int(n_samples)
    f64 = lambda a: (a if isinstance(a, torch.Tensor) else torch.as_tensor(np.asarray(a))).to(
        device=device, dtype=torch.float64).contiguous()
    lc, lm, li, ld = f64(log_chi), f64(log_M), f64(log_I), f64(log_D)
    if lc.dim() == 2:
        lc = lc.unsqueeze(0)
    res_t = torch.from_numpy(buf).to(device)
    b = DeviceBatch(Lx=Lx, Ly=Ly, x_off=xo, y_off=yo, residues=res_t, chi=lc, emit_M=lm, emit_I=li, emit_D=ld)
    bs = b.struct()
    nb = ctypes.c_size_t(0)
    _check(lib.phmm_sample_workspace_bytes(ctypes.byref(md), ctypes.byref(bs), ctypes.byref(nb)),
           'phmm_sample_workspace_bytes')
    ws = torch.empty(max(int(nb.value), 256), dtype=torch.uint8, device=device)
    ll = torch.empty(P, dtype=torch.float64, device=device)
    slots = (Lx.astype(np.int64) + Ly + 1)
    paths = torch.zeros(max(int(S * slots.sum()), 1), 3, dtype=torch.int32, device=device)
    plen = torch.zeros(max(P * S, 1), dtype=torch.int32, device=device)
    status = torch.zeros(P, dtype=torch.int32, device=device)
    s = stream if stream is not None else torch.cuda.current_stream(torch.device(device))
    _check(lib.phmm_sample_paths(ctypes.byref(md), ctypes.byref(bs), _ptr(lc), _ptr(lm), _ptr(li), _ptr(ld), S,
                                 ctypes.c_uint64(int(seed) & 0xFFFFFFFFFFFFFFFF), _ptr(ws),
                                 ctypes.c_size_t(ws.numel()), _ptr(ll), _ptr(paths), _ptr(plen), _ptr(status),
                                 ctypes.c_void_p(s.cuda_stream)), 'phmm_sample_paths')
    h = to_host({'ll': ll, 'paths': paths, 'plen': plen})
    offs = np.concatenate([[0], np.cumsum(S * slots)[:-1]])
    out = []
    for p in range(P):
        one = []
        for k in range(S):
            o = offs[p] + k * slots[p]
            one.append(h['paths'][o:o + h['plen'][p * S + k]])
        out.append(one)
    return h['ll'], out


def holmes_rubin(class_Q, class_pis, t, class_match_counts, stream=None, out=None):
    """phmm_holmes_rubin: (W [P,C,A], U [P,C,A,A]) float64 device tensors for
    host rate matrices class_Q [C,A,A], frequencies class_pis [C,A], device
    times t [P] and device match counts [P,C,A,A]."""
    lib = load()
    host = lambda v: v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else v
    Q = np.ascontiguousarray(np.asarray(host(class_Q), np.float64))
    pis = np.ascontiguousarray(np.asarray(host(class_pis), np.float64))
    if Q.ndim == 2:
        Q, pis = Q[None], pis.reshape(1, -1)
    C, A = pis.shape
    mc = class_match_counts.to(torch.float64).contiguous()
    P = mc.shape[0]
    tt = t.to(device=mc.device, dtype=torch.float64).reshape(-1).contiguous()
    if out is not None:
        W, U = out
    else:
        W = torch.empty(P, C, A, dtype=torch.float64, device=mc.device)
        U = torch.empty(P, C, A, A, dtype=torch.float64, device=mc.device)
    s = stream if stream is not None else torch.cuda.current_stream(mc.device)
    _check(lib.phmm_holmes_rubin(C, A, Q.ctypes.data, pis.ctypes.data, P, _ptr(tt), _ptr(mc), _ptr(W), _ptr(U),
                                 ctypes.c_void_p(s.cuda_stream)), 'phmm_holmes_rubin')
    return W, U


def fb1d(n_states, L, off, emit, chi, chi_per_pair, init_state, final_state, posteriors=False, stream=None):
    """phmm_fb1d: (ll [P] f64, n_trans [P,N,N] f64, posteriors [cols,N] f32 or None,
    status [P] i32) for per-pair column ranges of emit [cols, N] (device float32)."""
    lib = load()
    L = np.ascontiguousarray(np.asarray(L, np.int32))
    off = np.ascontiguousarray(np.asarray(off, np.int64))
    P = L.size
    dev = emit.device
    b = Fb1dBatch(P, n_states, L.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                  off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), emit.data_ptr(), chi.data_ptr(),
                  int(chi_per_pair), int(init_state), int(final_state))
    nb = ctypes.c_size_t(0)
    _check(lib.phmm_fb1d_workspace_bytes(ctypes.byref(b), ctypes.byref(nb)), 'phmm_fb1d_workspace_bytes')
    ws = torch.empty(max(int(nb.value), 256), dtype=torch.uint8, device=dev)
    ll = torch.empty(P, dtype=torch.float64, device=dev)
    nt = torch.empty(P, n_states, n_states, dtype=torch.float64, device=dev)
    st = torch.empty(P, dtype=torch.int32, device=dev)
    post = torch.zeros(emit.shape[0], n_states, dtype=torch.float32, device=dev) if posteriors else None
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _check(lib.phmm_fb1d(ctypes.byref(b), _ptr(ws), ctypes.c_size_t(ws.numel()), _ptr(ll), _ptr(nt), _ptr(post),
                         _ptr(st), ctypes.c_void_p(s.cuda_stream)), 'phmm_fb1d')
    return ll, nt, post, st


def fb1d_emissions(state_types, groups, G, L, off, cols, anc, desc, emit_M, emit_I, emit_D, per_pair,
                   stream=None):
    """phmm_fb1d_emissions: per-column emissions [cols, N] (device float32) of
    alignments (device uint8 cols / anc / desc) from the per-group tables."""
    lib = load()
    st_arr = np.ascontiguousarray(np.asarray(state_types, np.int8))
    gr = np.ascontiguousarray(np.asarray(groups, np.int32))
    desc_m = ModelDesc(st_arr.size, st_arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)),
                       gr.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), int(G))
    L = np.ascontiguousarray(np.asarray(L, np.int32))
    off = np.ascontiguousarray(np.asarray(off, np.int64))
    P = L.size
    dev = cols.device
    n_cols = int(cols.numel())
    out = torch.zeros(max(n_cols, 1), st_arr.size, dtype=torch.float32, device=dev)
    ws = torch.empty(max(16 * P, 256), dtype=torch.uint8, device=dev)
    status = torch.empty(max(P, 1), dtype=torch.int32, device=dev)
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _check(lib.phmm_fb1d_emissions(ctypes.byref(desc_m), P, L.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                   off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _ptr(cols), _ptr(anc),
                                   _ptr(desc), _ptr(emit_M), _ptr(emit_I), _ptr(emit_D), int(per_pair), _ptr(ws),
                                   ctypes.c_size_t(ws.numel()), _ptr(out), _ptr(status),
                                   ctypes.c_void_p(s.cuda_stream)), 'phmm_fb1d_emissions')
    return out, status


def viterbi(state_types, groups, G, xs, ys, log_chi, log_M, log_I, log_D, device='cuda', stream=None,
            envelopes=None):
    """phmm_viterbi: (ll [P] float64 numpy, paths: list of [n_p, 3] int32 arrays of
    (i, j, state)).  log_chi [P or 1, N, N] and the per-group log tables
    [P or 1, G, ...] are float64 (torch or numpy); envelopes: optional per-pair
    (Lx+1, Ly+1) boolean arrays (beam_viterbi_2d's band constraint)."""
    lib = load()
    st_arr = np.ascontiguousarray(np.asarray(state_types, np.int8))
    gr = np.ascontiguousarray(np.asarray(groups, np.int32))
    md = ModelDesc(st_arr.size, st_arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)),
                   gr.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), int(G))
    buf, xo, yo, Lx, Ly = pack_residues(xs, ys)
    P = Lx.size
    f64 = lambda a: (a if isinstance(a, torch.Tensor) else torch.as_tensor(np.asarray(a))).to(
        device=device, dtype=torch.float64).contiguous()
    lc, lm, li, ld = f64(log_chi), f64(log_M), f64(log_I), f64(log_D)
    if lc.dim() == 2:
        lc = lc.unsqueeze(0)
    res_t = torch.from_numpy(buf).to(device)
    env = None
    if envelopes is not None:
        env = torch.from_numpy(np.concatenate([np.asarray(e, bool).reshape(-1) for e in envelopes]).astype(
            np.uint8)).to(device)
    b = DeviceBatch(Lx=Lx, Ly=Ly, x_off=xo, y_off=yo, residues=res_t, chi=lc, emit_M=lm, emit_I=li, emit_D=ld,
                    cell_mask=env)
    bs = b.struct()
    nb = ctypes.c_size_t(0)
    _check(lib.phmm_viterbi_workspace_bytes(ctypes.byref(md), ctypes.byref(bs), ctypes.byref(nb)),
           'phmm_viterbi_workspace_bytes')
    ws = torch.empty(max(int(nb.value), 256), dtype=torch.uint8, device=device)
    ll = torch.empty(P, dtype=torch.float64, device=device)
    n_path = int(np.sum(Lx.astype(np.int64) + Ly + 1))
    path = torch.zeros(max(n_path, 1), 3, dtype=torch.int32, device=device)
    plen = torch.zeros(P, dtype=torch.int32, device=device)
    status = torch.zeros(P, dtype=torch.int32, device=device)
    s = stream if stream is not None else torch.cuda.current_stream(torch.device(device))
    _check(lib.phmm_viterbi(ctypes.byref(md), ctypes.byref(bs), _ptr(lc), _ptr(lm), _ptr(li), _ptr(ld), _ptr(ws),
                            ctypes.c_size_t(ws.numel()), _ptr(ll), _ptr(path), _ptr(plen), _ptr(status),
                            ctypes.c_void_p(s.cuda_stream)), 'phmm_viterbi')
    ll_h, path_h, plen_h = ll.cpu().numpy(), path.cpu().numpy(), plen.cpu().numpy()
    offs = np.concatenate([[0], np.cumsum(Lx.astype(np.int64) + Ly + 1)[:-1]])
    return ll_h, [path_h[o:o + n] for o, n in zip(offs, plen_h)]
