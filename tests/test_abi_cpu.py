"""CPU-side checks of the C ABI: the library builds, loads, exports every
symbol that include/pairhmm.h declares, and rejects bad model descriptions
without touching a GPU."""
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, 'include', 'pairhmm.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(phmm_[a-z0-9_]+)\s*\(', src)))


@pytest.fixture(scope='module')
def lib():
    from pairhmm import build, _lib
    build.build()
    return _lib.load()


def test_header_declares_the_abi():
    syms = declared_symbols()
    from pairhmm import _lib
    assert set(syms) == set(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_version_and_error_reporting(lib):
    assert lib.phmm_version() == 1
    import ctypes
    from pairhmm import _lib
    # a model whose state 0 is not the start state is rejected before any CUDA call
    desc = _lib.ModelDesc(3, (ctypes.c_int8 * 3)(1, 2, 4), None, 1)
    h = ctypes.c_void_p()
    rc = lib.phmm_plan_create(ctypes.byref(desc), ctypes.byref(h))
    assert rc == -1
    assert 'start' in _lib.last_error()
    desc = _lib.ModelDesc(3, (ctypes.c_int8 * 3)(0, 1, 2), None, 1)
    assert lib.phmm_plan_create(ctypes.byref(desc), ctypes.byref(h)) == -1
    assert 'End' in _lib.last_error()


def test_mixdom2_prologue_rejects_bad_shapes(lib):
    """phmm_mixdom2_tables checks the parameter shapes before any CUDA call."""
    import ctypes
    import numpy as np
    from pairhmm import _lib
    K, F, C = 8, 5, 1
    arrs = [np.ones(n) for n in (K, K, K, K * F, K * F * F, C * 20, C * 400, K * F * C)]
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    prm = _lib.MixDom2Params(K, F, C, 20, 0.03, 0.04, *[dp(a) for a in arrs])
    null = ctypes.c_void_p(0)
    assert lib.phmm_mixdom2_tables(ctypes.byref(prm), 4, *([null] * 7)) == -1
    assert '33' in _lib.last_error()
    prm = _lib.MixDom2Params(2, 1, 1, 4, 0.03, 0.04, *[dp(a) for a in arrs])
    assert lib.phmm_mixdom2_tables(ctypes.byref(prm), 4, *([null] * 7)) == -1
    assert 'alphabet' in _lib.last_error()
    prm = _lib.MixDom2Params(2, 1, 1, 20, 0.03, 0.04, *[dp(a) for a in arrs])
    assert lib.phmm_mixdom2_tables(ctypes.byref(prm), 4, *([null] * 7)) == -1
    assert 'null device buffer' in _lib.last_error()
    assert lib.phmm_mixdom2_tables(ctypes.byref(prm), 0, *([null] * 7)) == 0
    assert lib.phmm_mixdom2_class_subs_count(ctypes.byref(prm), 10) == 10 * 400


def test_holmes_rubin_rejects_bad_arguments(lib):
    """phmm_holmes_rubin checks its arguments before any CUDA call."""
    import ctypes
    import numpy as np
    from pairhmm import _lib
    Q = np.zeros((1, 4, 4))
    pi = np.full((1, 4), 0.25)
    null = ctypes.c_void_p(0)
    assert lib.phmm_holmes_rubin(1, 40, Q.ctypes.data, pi.ctypes.data, 3, null, null, null, null, null) == -1
    assert 'alphabet' in _lib.last_error()
    bad = np.array([[0.5, 0.5, 0.0, 0.0]])
    assert lib.phmm_holmes_rubin(1, 4, Q.ctypes.data, bad.ctypes.data, 3, null, null, null, null, null) == -1
    assert 'positive' in _lib.last_error()
    assert lib.phmm_holmes_rubin(1, 4, Q.ctypes.data, pi.ctypes.data, 3, null, null, null, null, null) == -1
    assert 'null device buffer' in _lib.last_error()
    assert lib.phmm_holmes_rubin(1, 4, Q.ctypes.data, pi.ctypes.data, 0, null, null, null, null, null) == 0


def test_sample_paths_rejects_bad_arguments(lib):
    """phmm_sample_paths checks its arguments before any CUDA call."""
    import ctypes
    import numpy as np
    from pairhmm import _lib
    st = (ctypes.c_int8 * 5)(0, 1, 2, 3, 4)
    gr = (ctypes.c_int32 * 5)(0, 0, 0, 0, 0)
    desc = _lib.ModelDesc(5, st, gr, 1)
    Lx = np.array([3], np.int32)
    Ly = np.array([4], np.int32)
    off = np.array([0], np.int64)
    b = _lib.Batch(1, Lx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), Ly.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                   None, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                   off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), None, 0, None, None, None, 0, None, 0.0)
    null = ctypes.c_void_p(0)
    args = [null] * 4 + [8, 1, null, 0, null, null, null, null, null]
    assert lib.phmm_sample_paths(ctypes.byref(desc), ctypes.byref(b), *args) == -1
    assert 'null pointer' in _lib.last_error()
    bad = [null] * 4 + [-1, 1, null, 0, null, null, null, null, null]
    assert lib.phmm_sample_paths(ctypes.byref(desc), ctypes.byref(b), *bad) == -1
    assert 'negative' in _lib.last_error()
    big = _lib.ModelDesc(70, (ctypes.c_int8 * 70)(*([0] + [1] * 68 + [4])), (ctypes.c_int32 * 70)(), 1)
    assert lib.phmm_sample_paths(ctypes.byref(big), ctypes.byref(b), *args) == -1
    assert '2..64' in _lib.last_error()
    nb = ctypes.c_size_t(0)
    assert lib.phmm_sample_workspace_bytes(ctypes.byref(desc), ctypes.byref(b), ctypes.byref(nb)) == 0
    assert nb.value >= 4 * 5 * 5 * 8


def test_static_estep_refuses_masks_and_beam(lib):
    """phmm_estep_static has no cell-mask or beam support and says so before
    any CUDA call."""
    import ctypes
    import numpy as np
    from pairhmm import _lib
    st = (ctypes.c_int8 * 5)(0, 1, 2, 3, 4)
    gr = (ctypes.c_int32 * 5)(0, 0, 0, 0, 0)
    desc = _lib.ModelDesc(5, st, gr, 1)
    Lx = np.array([3], np.int32)
    off = np.array([0], np.int64)
    dummy = np.zeros(64, np.float64)      # host memory standing in for device pointers: never read
    vp = ctypes.c_void_p(dummy.ctypes.data)
    i32 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    i64 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    for mask, beam, word in ((vp, 0.0, 'cell masks'), (None, 2.0, 'beam')):
        b = _lib.Batch(1, i32(Lx), i32(Lx), vp, i64(off), i64(off), vp, 0, vp, vp, vp, 0, mask, beam)
        rc = lib.phmm_estep_static(ctypes.byref(desc), ctypes.byref(b), *([vp] * 6), None)
        assert rc == -1 and word in _lib.last_error()


def test_fb1d_and_viterbi_and_pairs_reject_bad_arguments(lib):
    """Argument checks of the 1D forward-backward, Viterbi and record-reader
    entries, all before any CUDA call."""
    import ctypes
    import numpy as np
    from pairhmm import _lib, pair_format as pf
    null = ctypes.c_void_p(0)
    L = np.array([3], np.int32)
    off = np.array([0], np.int64)
    b = _lib.Fb1dBatch(1, 70, L.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                       off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), None, None, 0, 0, 1)
    assert lib.phmm_fb1d(ctypes.byref(b), null, 0, null, null, null, null, null) == -1
    assert '2..64' in _lib.last_error()
    b.n_states = 5
    b.final_state = 9
    assert lib.phmm_fb1d(ctypes.byref(b), null, 0, null, null, null, null, null) == -1
    assert 'final state' in _lib.last_error()
    b.final_state = 4
    assert lib.phmm_fb1d(ctypes.byref(b), null, 0, null, null, null, null, null) == -1
    assert 'null pointer' in _lib.last_error()
    b.n_pairs = 0
    assert lib.phmm_fb1d(ctypes.byref(b), null, 0, null, null, null, null, null) == 0
    # Viterbi: state 0 must be S and one state E
    st = (ctypes.c_int8 * 3)(1, 2, 3)
    gr = (ctypes.c_int32 * 3)(0, 0, 0)
    desc = _lib.ModelDesc(3, st, gr, 1)
    Lx = np.array([2], np.int32)
    dummy = np.zeros(16)
    vp = ctypes.c_void_p(dummy.ctypes.data)
    i32 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    i64 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    bt = _lib.Batch(1, i32(Lx), i32(Lx), vp, i64(off), i64(off), vp, 0, vp, vp, vp, 0, None, 0.0)
    wsbuf = np.zeros(1024, np.uint8)
    ws = ctypes.c_void_p((wsbuf.ctypes.data + 255) & ~255)   # 256-byte aligned, never read
    args = [vp] * 4 + [ws, ctypes.c_size_t(512), vp, vp, vp, vp, null]
    assert lib.phmm_viterbi(ctypes.byref(desc), ctypes.byref(bt), *args) == -1
    assert 'state 0 must be S' in _lib.last_error()
    # record reader: sizes that do not match the text
    cnt = pf.PairCounts(2, 4, 2)
    pf._bind(lib)
    one = b'{"x": "AC", "a": "M2", "y": "AC", "t": 1}\n'
    arrs = [np.zeros(8, np.int64) for _ in range(13)]
    rc = lib.phmm_pairs_decode(one, len(one), ctypes.byref(cnt), *[ctypes.c_void_p(a.ctypes.data) for a in arrs])
    assert rc == -1 and 'less than the counted sizes' in _lib.last_error()
