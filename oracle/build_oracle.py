"""Build the C half of the oracle (TEST INFRASTRUCTURE ONLY): oracle/fb2d.c
compiled with the host C compiler into oracle/_build/liboracle.so, with
OpenMP where the compiler has it (serial otherwise).  Called by
__graft_entry__.build(); skipped when the library is newer than its source."""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'fb2d.c')
LIB = os.path.join(HERE, '_build', 'liboracle.so')


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cc = os.environ.get('CC') or shutil.which('gcc') or shutil.which('cc')
    if not cc:
        raise RuntimeError('no C compiler for the oracle')
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + '.tmp'
    base = [cc, '-O2', '-fPIC', '-shared', '-std=c99', SRC, '-o', tmp]
    res = subprocess.run(base[:1] + ['-fopenmp'] + base[1:] + ['-lm'], capture_output=True, text=True)
    if res.returncode != 0:   # no OpenMP runtime: the serial build
        subprocess.run(base + ['-lm'], check=True, capture_output=True, text=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force=True))
