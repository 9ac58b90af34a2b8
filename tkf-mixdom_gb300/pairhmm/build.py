"""In-tree build of the CUDA library (``libpairhmm.so``) for sm_103a.

``python -m pairhmm.build`` (or ``build()``) compiles the translation units
of ``csrc/`` (the E-step kernels and C ABI in ``pairhmm.cu``, the device
prologue in ``prologue.cu``, the 1D alignment-conditioned forward-backward in
``fb1d.cu``, the Viterbi decoder in ``viterbi.cu``, the path sampler in
``sample.cu``, the pair-record reader in ``pairs.cpp``) in parallel with nvcc and links them into
``pairhmm/libpairhmm.so`` next to this file.  The build is skipped when the
library is newer than its sources.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
PROJECT_DIR = os.path.dirname(PKG_DIR)
REPO_DIR = os.path.dirname(PROJECT_DIR)
CSRC = os.path.join(PROJECT_DIR, 'csrc')
INCLUDE = os.path.join(REPO_DIR, 'include')
LIB_PATH = os.path.join(PKG_DIR, 'libpairhmm.so')
SOURCES = [os.path.join(CSRC, f) for f in ('pairhmm.cu', 'prologue.cu', 'fb1d.cu', 'viterbi.cu', 'sample.cu', 'pairs.cpp')]
OBJ_DIR = os.path.join(PKG_DIR, '_build')
ARCH_FLAGS = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc_path():
    cand = shutil.which('nvcc')
    if cand:
        return cand
    for p in ('/usr/local/cuda/bin/nvcc',):
        if os.path.exists(p):
            return p
    raise RuntimeError('nvcc not found')


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    deps = SOURCES + [os.path.join(INCLUDE, 'pairhmm.h')] + [
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
    if not force and not _stale(LIB_PATH, deps):
        return LIB_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = nvcc_path()
    procs = []
    for src in SOURCES:
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + '.o')
        cmd = [nvcc, *ARCH_FLAGS, '-O3', '-lineinfo', '-std=c++17', '-c', '-Xcompiler', '-fPIC',
               '-I', INCLUDE, *extra, src, '-o', obj]
        if verbose:
            print(' '.join(cmd), file=sys.stderr)
        procs.append((obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)))
    objs, errors = [], []
    for obj, pr in procs:
        out, err = pr.communicate()
        if pr.returncode != 0:
            errors.append(out + err)
        elif verbose and err:
            print(err, file=sys.stderr)
        objs.append(obj)
    if errors:
        raise RuntimeError('nvcc failed:\n' + '\n'.join(errors))
    tmp = LIB_PATH + '.tmp'
    cmd = [nvcc, *ARCH_FLAGS, '-shared', *objs, '-o', tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('nvcc link failed:\n' + res.stdout + res.stderr)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == '__main__':
    build(force='--force' in sys.argv, verbose=True,
          extra=['-Xptxas', '-v'] if '--ptxas' in sys.argv else ())
