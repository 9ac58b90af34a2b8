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
    return sorted(set(re.findall(r'\b(phmm_[a-z_]+)\s*\(', src)))


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
