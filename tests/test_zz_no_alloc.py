"""The allocation-free E-step entry point (phmm_estep_static).

It exists for callers whose process already owns the GPU memory (a JAX
runtime that reserved most of the device, a serving framework's allocator):
they cannot let this library cudaMalloc scratch.  The entry point runs the
E-step kernels on a fixed file-scope device array instead.  This test calls
it through the C ABI, twice in a row, and checks each result against the FP64
oracle and against phmm_estep (which allocates its scratch through a plan),
with the bars the other GPU tests use; it checks that repeated calls,
including a larger batch that still fits, leave the device's free memory
unchanged; and that an oversized batch is refused with a clear message.  The
file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
LL_RTOL = 1e-6
CNT_RTOL = 1e-5


def _model_and_batch(n_pairs, max_len, seed, fixed_len=None, with_oracle=False):
    import torch
    from pairhmm import _lib, synth
    from pairhmm import models as pm
    rng = np.random.default_rng(seed)
    p = synth.mixdom2_params(rng, 3, 1, 1)
    ts = np.exp(rng.uniform(np.log(0.05), np.log(2.0), n_pairs))
    ln = (lambda: fixed_len) if fixed_len else (lambda: int(rng.integers(0, max_len)))
    xs = [rng.integers(0, 20, ln()) for _ in range(n_pairs)]
    ys = [rng.integers(0, 20, ln()) for _ in range(n_pairs)]
    chi = pm.build_nested_trans(p['main_ins'], p['main_del'], torch.as_tensor(ts), p['dom_ins'],
                                p['dom_del'], p['dom_weights'], p['frag_weights'], p['ext_rates'])
    cs = pm.class_subs(p['class_S_exch'], p['class_pis'], torch.as_tensor(ts))
    EM, EI, ED = pm.tables_per_class(cs, p['class_pis'], p['classdist'])
    st = pm.mixdom_state_types(3, 1)
    gr = pm.mixdom_state_groups(3, 1)
    batch = _lib.make_batch(xs, ys, chi, EM, EI, ED, device='cuda')
    if not with_oracle:
        return st, gr, batch
    from oracle import estep as oe, pool
    cases = []
    for b in range(n_pairs):
        ochi, ost, ogr, oEM, oEI, oED, _ = oe.mixdom2_model(dict(p, t=float(ts[b])))
        cases.append((ochi, ost, ogr, oEM, oEI, oED, xs[b], ys[b]))
    return st, gr, batch, pool.estep_pairs(cases)


def _outputs(P, N, G):
    import torch
    dev = 'cuda'
    return {'ll': torch.empty(P, dtype=torch.float64, device=dev),
            'n_trans': torch.empty(P, N, N, dtype=torch.float64, device=dev),
            'cnt_M': torch.empty(P, G, 21, 21, dtype=torch.float64, device=dev),
            'cnt_I': torch.empty(P, G, 21, dtype=torch.float64, device=dev),
            'cnt_D': torch.empty(P, G, 21, dtype=torch.float64, device=dev),
            'status': torch.empty(P, dtype=torch.int32, device=dev)}


def _static_call(lib, st, gr, G, batch, out):
    import torch
    from pairhmm import _lib
    st8 = np.ascontiguousarray(st, dtype=np.int8)
    gr32 = np.ascontiguousarray(gr, dtype=np.int32)
    desc = _lib.ModelDesc(st8.size, st8.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)),
                          gr32.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), G)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.phmm_estep_static(ctypes.byref(desc), ctypes.byref(batch.struct()), p(out['ll']),
                               p(out['n_trans']), p(out['cnt_M']), p(out['cnt_I']), p(out['cnt_D']),
                               p(out['status']), stream)
    return rc


def _close(got, want, rtol):
    got = got.cpu().numpy()
    want = want.cpu().numpy()
    scale = max(np.abs(want).max(), 1e-300)
    assert np.abs(got - want).max() <= rtol * scale + 1e-12


def test_static_estep_matches_oracle_and_plan_estep_twice(cuda_lib):
    import torch
    from pairhmm import _lib
    from oracle import pool
    lib = cuda_lib
    st, gr, batch, oracle = _model_and_batch(12, 120, seed=4, with_oracle=True)
    N, G = len(st), 3
    plan = _lib.Plan(st, gr, G)
    want = _lib.estep(plan, batch)
    torch.cuda.synchronize()
    for call in range(2):
        out = _outputs(batch.n_pairs, N, G)
        for v in out.values():
            v.fill_(7)   # stale contents must not leak into the result
        rc = _static_call(lib, st, gr, G, batch, out)
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        assert (out['status'] == 0).all()
        ll, llw = out['ll'].cpu().numpy(), want['ll'].cpu().numpy()
        assert np.all(np.abs(ll - llw) <= LL_RTOL * np.abs(llw)), call
        for k in ('n_trans', 'cnt_M', 'cnt_I', 'cnt_D'):
            _close(out[k], want[k], CNT_RTOL)
        # and against the FP64 oracle, pair by pair
        host = {k: v.cpu().numpy() for k, v in out.items()}
        for b, (oll, n, cnt) in enumerate(oracle):
            assert abs(host['ll'][b] - oll) <= LL_RTOL * abs(oll), (call, b, host['ll'][b], oll)
            for key, w in zip(('n_trans', 'cnt_M', 'cnt_I', 'cnt_D'), (n, *cnt)):
                abs_of_max, rel = pool.count_errors(host[key][b], w)
                assert abs_of_max <= CNT_RTOL and rel < CNT_RTOL, (call, b, key, abs_of_max, rel)


def test_static_estep_allocates_nothing(cuda_lib):
    """After a first call (which loads the kernels and looks the array up),
    further calls -- among them a larger batch that still fits -- leave the
    device's free memory exactly where it was."""
    import torch
    from pairhmm import _lib
    lib = cuda_lib
    st, gr, small = _model_and_batch(6, 90, seed=8)
    _, _, large = _model_and_batch(10, 0, seed=9, fixed_len=150)   # about 410 k stripe cells
    N, G = len(st), 3
    outs = [_outputs(small.n_pairs, N, G), _outputs(large.n_pairs, N, G)]
    assert _static_call(lib, st, gr, G, small, outs[0]) == 0, _lib.last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for batch, out in ((large, outs[1]), (small, outs[0]), (large, outs[1])):
        assert _static_call(lib, st, gr, G, batch, out) == 0, _lib.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert (outs[1]['status'] == 0).all() and torch.isfinite(outs[1]['ll']).all()


def test_static_estep_refuses_oversized_batch(cuda_lib):
    from pairhmm import _lib
    lib = cuda_lib
    # four 3000 x 3000 pairs need ~2.4 GB of scratch: refused before any kernel runs
    st, gr, batch = _model_and_batch(4, 0, seed=1, fixed_len=3000)
    out = _outputs(4, len(st), 3)
    rc = _static_call(lib, st, gr, 3, batch, out)
    assert rc == -1
    msg = _lib.last_error()
    assert 'bytes of scratch' in msg and str(32 * 1024 * 1024) in msg
