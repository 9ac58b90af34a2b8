"""The serving loop on the GPU: each request's result is the same alone and
in a mixed stream (continuous batching, several batches in flight, three
models), and the same as the batched API and the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
LL_RTOL = 1e-6
CNT_RTOL = 1e-5
KEYS = ('n_trans', 'cnt_M', 'cnt_I', 'cnt_D')


def _stream(n, seed, hi=300):
    from pairhmm import synth
    return synth.make_serving_stream(n, rate=5000.0, law=('loguniform', 20, hi), seed=seed)


def _server(models, **kw):
    from pairhmm.serving import Server, ServedModel
    return Server([ServedModel(name, kind, p) for name, (kind, p) in models.items()], **kw)


def _requests(reqs):
    from pairhmm.serving import Request
    return [Request(i, m, x, y, t) for i, (m, x, y, t) in enumerate(reqs)]


def _close_counts(a, b, what):
    for k in KEYS + tuple(k for k in a if k.startswith('class')):
        scale = max(np.abs(b[k]).max(), 1e-300)
        err = np.abs(a[k] - b[k]).max()
        assert err <= CNT_RTOL * scale + 1e-12, (what, k, err / scale)


def _alone(models, reqs, **kw):
    srv = _server(models, max_inflight=1, max_batch=1, **kw)
    out = []
    for r in _requests(reqs):
        srv.submit(r)
        srv.drain()
        assert r.error is None, r.error
        out.append(r)
    return out


def test_results_equal_alone_and_in_mixed_stream(cuda_lib):
    from pairhmm.serving import latency_summary, run_stream
    models, reqs, offsets = _stream(36, seed=3)
    alone = _alone(models, reqs, arena_bytes=256 << 20)
    srv = _server(models, arena_bytes=256 << 20, max_inflight=4, max_batch=8)
    mixed, wall = run_stream(srv.sched, _requests(reqs), offsets)
    summ = latency_summary(mixed, wall)
    assert summ['completed'] == len(reqs) and summ['failed'] == 0
    assert srv.sched.batches < len(reqs)             # requests were batched together
    assert max(srv.sched.batch_sizes) > 1
    assert {r.model for r in mixed} == set(models)
    for a, m in zip(alone, mixed):
        la, lm = float(a.result['log_p']), float(m.result['log_p'])
        assert abs(la - lm) <= LL_RTOL * abs(la), (a.rid, la, lm)
        assert int(m.result['status']) == 0
        _close_counts(m.result, a.result, a.rid)


def test_tight_arena_serialises_but_keeps_results(cuda_lib):
    models, reqs, offsets = _stream(12, seed=5, hi=200)
    srv = _server(models, arena_bytes=256 << 20, max_inflight=4, max_batch=8)
    need = max(srv.executor.request_bytes(r) for r in _requests(reqs))
    tight = _server(models, arena_bytes=need + 4096, max_inflight=4, max_batch=8)
    got = _requests(reqs)
    for r in got:
        tight.submit(r)
    tight.drain()
    assert tight.sched.peak_bytes <= need + 4096
    alone = _alone(models, reqs, arena_bytes=256 << 20)
    for a, m in zip(alone, got):
        assert m.error is None, m.error
        la, lm = float(a.result['log_p']), float(m.result['log_p'])
        assert abs(la - lm) <= LL_RTOL * abs(la)
        _close_counts(m.result, a.result, a.rid)


def test_served_results_match_batched_api_and_oracle(cuda_lib):
    from pairhmm import api
    from oracle import estep as oe
    models, reqs, _ = _stream(24, seed=7, hi=150)
    srv = _server(models, arena_bytes=256 << 20, max_inflight=3, max_batch=6)
    got = _requests(reqs)
    for r in got:
        srv.submit(r)
    srv.drain()
    name = 'mixdom2_k3f1c1'
    kind, params = models[name]
    sel = [r for r in got if r.model == name]
    assert sel
    ref = api.estep_batch_mixdom2(params, [r.x for r in sel], [r.y for r in sel],
                                  np.array([r.t for r in sel]))
    for k, r in enumerate(sel):
        lr = float(ref['log_p'][k])
        assert abs(float(r.result['log_p']) - lr) <= LL_RTOL * abs(lr)
        for key in ('n_trans', 'cnt_M', 'class_match_counts', 'classdist_counts'):
            want = ref[key][k].cpu().numpy()
            assert np.abs(r.result[key] - want).max() <= CNT_RTOL * max(np.abs(want).max(), 1e-300) + 1e-12
    # one short request per model against the float64 oracle
    for name, (kind, params) in models.items():
        r = min((q for q in got if q.model == name), key=lambda q: len(q.x) * len(q.y))
        if kind == 'tkf92':
            p = dict(params, t=r.t)
            ll, n_tr, _ = oe.e_step('tkf92', p, r.x, r.y)
        else:
            p = dict(params, t=r.t)
            ll, n_tr, _ = oe.e_step_mixdom2(p, r.x, r.y)
        assert abs(float(r.result['log_p']) - ll) <= LL_RTOL * abs(ll), name
        assert np.abs(r.result['n_trans'] - n_tr).max() <= CNT_RTOL * np.abs(n_tr).max() + 1e-12, name
