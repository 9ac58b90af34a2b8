"""A NumPy implementation of the small subset of the JAX API that the
reference pair-HMM modules use, so that those unmodified modules can be run
on the CPU (JAX is not installable in this environment).

Only used by ``make_golden.py`` to produce the golden fixtures; nothing in
the product or the GPU tests imports it.

Semantics reproduced (with x64 enabled, as the reference requires):
  * arrays are float64/int64 NumPy arrays with a functional ``.at[]``
    (set / add / multiply / min / max / get);
  * integer-array gathers clamp out-of-range indices (JAX's default gather
    mode), scatters into a copy;
  * jit / checkpoint / custom_vjp are identity wrappers (forward values only;
    a custom VJP's fwd / bwd functions are called directly by the fixture
    scripts);
  * grad is a Richardson-extrapolated central difference, for the closed-form
    functions that the reference's VJP backward passes differentiate;
  * vmap / lax.scan / lax.fori_loop are Python loops with pytree stacking;
  * nn.logsumexp follows JAX's max-shift formula; nn.one_hot drops
    out-of-range classes.
"""
from __future__ import annotations

import sys
import types
import functools

import numpy as np
import scipy.linalg
import scipy.special


class JArr(np.ndarray):
    """ndarray with JAX's functional ``.at`` updates and clamped gathers."""

    def __array_finalize__(self, obj):
        pass

    @property
    def at(self):
        return _At(self)

    def __getitem__(self, idx):
        return _wrap(np.ndarray.__getitem__(self.view(np.ndarray),
                                            _clamp_index(self.shape, idx)))


def _wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, JArr):
        return x.view(JArr)
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, list):
        return [_wrap(v) for v in x]
    return x


def _is_int_array(v):
    return (isinstance(v, (np.ndarray, np.integer))
            and np.asarray(v).dtype.kind in 'iu')


def _clamp_index(shape, idx):
    if not isinstance(idx, tuple):
        idx = (idx,)
    consumed = 0
    for v in idx:
        if v is None or v is Ellipsis:
            continue
        if isinstance(v, np.ndarray) and v.dtype == bool:
            consumed += v.ndim
        else:
            consumed += 1
    out = []
    dim = 0
    for v in idx:
        if v is Ellipsis:
            dim += len(shape) - consumed
            out.append(v)
            continue
        if v is None:
            out.append(v)
            continue
        if isinstance(v, np.ndarray) and v.dtype == bool:
            dim += v.ndim
            out.append(v.view(np.ndarray))
            continue
        if _is_int_array(v):
            n = shape[dim]
            a = np.asarray(v).astype(np.int64)
            a = np.where(a < 0, a + n, a)
            out.append(np.clip(a, 0, n - 1))
        elif isinstance(v, np.ndarray):
            out.append(v.view(np.ndarray))
        else:
            out.append(v)
        dim += 1
    return tuple(out)


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIdx(self.arr, idx)


class _AtIdx:
    def __init__(self, arr, idx):
        self.arr = arr
        self.idx = idx

    def _copy(self, v):
        base = np.array(self.arr, copy=True).view(np.ndarray)
        vv = np.asarray(v)
        if vv.dtype.kind == 'f' and base.dtype.kind in 'iub':
            base = base.astype(np.float64)
        return base, vv

    def _index(self):
        idx = self.idx if isinstance(self.idx, tuple) else (self.idx,)
        return tuple(np.asarray(v).view(np.ndarray) if isinstance(v, np.ndarray) else v
                     for v in idx)

    def set(self, v, **_):
        base, vv = self._copy(v)
        base[self._index()] = vv
        return base.view(JArr)

    def add(self, v, **_):
        base, vv = self._copy(v)
        np.add.at(base, self._index(), vv)
        return base.view(JArr)

    def multiply(self, v, **_):
        base, vv = self._copy(v)
        np.multiply.at(base, self._index(), vv)
        return base.view(JArr)

    def min(self, v, **_):
        base, vv = self._copy(v)
        np.minimum.at(base, self._index(), vv)
        return base.view(JArr)

    def max(self, v, **_):
        base, vv = self._copy(v)
        np.maximum.at(base, self._index(), vv)
        return base.view(JArr)

    def get(self, **_):
        return self.arr[self.idx]


def _wrap_fn(fn):
    @functools.wraps(fn)
    def inner(*a, **k):
        k.pop('precision', None)
        return _wrap(fn(*a, **k))
    return inner


def _module_proxy(name, source, overrides=None):
    mod = types.ModuleType(name)
    overrides = overrides or {}

    def __getattr__(attr):
        if attr in overrides:
            return overrides[attr]
        obj = getattr(source, attr)
        if callable(obj) and not isinstance(obj, type):
            return _wrap_fn(obj)
        return obj
    mod.__getattr__ = __getattr__
    for k, v in overrides.items():
        setattr(mod, k, v)
    return mod


# ---------------------------------------------------------------- jax.numpy
def _asarray(x, dtype=None, **_):
    return _wrap(np.asarray(x, dtype=dtype))


def _array(x, dtype=None, **_):
    return _wrap(np.array(x, dtype=dtype))


jnp = _module_proxy('jax.numpy', np, {
    'asarray': _asarray,
    'array': _array,
    'ndarray': np.ndarray,
})
jnp.linalg = _module_proxy('jax.numpy.linalg', np.linalg)


# ---------------------------------------------------------------- jax.nn
def logsumexp(a, axis=None, b=None, keepdims=False, return_sign=False):
    a = np.asarray(a, dtype=np.float64)
    amax = np.max(a, axis=axis, keepdims=True)
    amax = np.where(np.isfinite(amax), amax, 0.0)
    ex = np.exp(a - amax)
    if b is not None:
        ex = ex * np.asarray(b)
    s = np.sum(ex, axis=axis, keepdims=True)
    with np.errstate(divide='ignore'):
        out = np.log(s) + amax
    if not keepdims:
        out = np.squeeze(out, axis=axis) if axis is not None else out.reshape(())
    return _wrap(np.asarray(out))


def one_hot(x, num_classes, dtype=np.float64, **_):
    x = np.asarray(x)
    return _wrap((x[..., None] == np.arange(num_classes)).astype(dtype))


nn = types.ModuleType('jax.nn')
nn.logsumexp = logsumexp
nn.one_hot = one_hot
nn.softmax = _wrap_fn(lambda a, axis=-1: np.exp(a - scipy.special.logsumexp(a, axis=axis, keepdims=True)))


# ---------------------------------------------------------------- pytrees
def _tree_leaves_stack(items):
    first = items[0]
    if first is None:
        return None
    if isinstance(first, tuple):
        return tuple(_tree_leaves_stack([it[i] for it in items]) for i in range(len(first)))
    if isinstance(first, list):
        return [_tree_leaves_stack([it[i] for it in items]) for i in range(len(first))]
    if isinstance(first, dict):
        return {k: _tree_leaves_stack([it[k] for it in items]) for k in first}
    return _wrap(np.stack([np.asarray(it) for it in items]))


def _tree_index(tree, i):
    if tree is None:
        return None
    if isinstance(tree, tuple):
        return tuple(_tree_index(t, i) for t in tree)
    if isinstance(tree, list):
        return [_tree_index(t, i) for t in tree]
    if isinstance(tree, dict):
        return {k: _tree_index(v, i) for k, v in tree.items()}
    return _wrap(np.asarray(tree)[i])


def _tree_len(tree):
    if isinstance(tree, (tuple, list)):
        for t in tree:
            n = _tree_len(t)
            if n is not None:
                return n
        return None
    if isinstance(tree, dict):
        for t in tree.values():
            n = _tree_len(t)
            if n is not None:
                return n
        return None
    if tree is None:
        return None
    return np.asarray(tree).shape[0]


# ---------------------------------------------------------------- jax.lax
def scan(f, init, xs=None, length=None, reverse=False, **_):
    n = length if xs is None else _tree_len(xs)
    order = range(n - 1, -1, -1) if reverse else range(n)
    carry = init
    ys = []
    for i in order:
        carry, y = f(carry, None if xs is None else _tree_index(xs, i))
        ys.append(y)
    if reverse:
        ys = ys[::-1]
    if not ys or ys[0] is None:
        return carry, None
    return carry, _tree_leaves_stack(ys)


def fori_loop(lo, hi, body, init, **_):
    v = init
    for i in range(int(lo), int(hi)):
        v = body(i, v)
    return v


def cond(pred, tf, ff, *ops, **_):
    return tf(*ops) if bool(pred) else ff(*ops)


def dynamic_slice(operand, start_indices, slice_sizes):
    """jax.lax.dynamic_slice: start indices clamped so the slice stays inside."""
    a = np.asarray(operand)
    idx = []
    for dim, st, n in zip(a.shape, start_indices, slice_sizes):
        st = int(min(max(int(st), 0), dim - int(n)))
        idx.append(slice(st, st + int(n)))
    return _wrap(a[tuple(idx)])


def associative_scan(fn, elems, reverse=False, axis=0):
    """jax.lax.associative_scan as a sequential inclusive scan along axis 0
    (the reduction order of a prefix scan; fn is associative)."""
    if axis != 0:
        raise NotImplementedError('associative_scan stand-in: axis 0 only')
    n = _tree_len(elems)
    order = range(n - 1, -1, -1) if reverse else range(n)
    out = [None] * n
    acc = None
    for i in order:
        e = _tree_index(elems, i)
        acc = e if acc is None else (fn(e, acc) if reverse else fn(acc, e))
        out[i] = acc
    return _tree_leaves_stack(out)


lax = types.ModuleType('jax.lax')
lax.scan = scan
lax.fori_loop = fori_loop
lax.cond = cond
lax.stop_gradient = lambda x: x
lax.dynamic_slice = dynamic_slice
lax.associative_scan = associative_scan


# ---------------------------------------------------------------- transforms
def jit(f=None, **_):
    if f is None:
        return lambda g: g
    return f


def vmap(f, in_axes=0, out_axes=0, **_):
    def inner(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = None
        for a, ax in zip(args, axes):
            if ax is not None:
                n = _tree_len(a)
                break
        outs = []
        for i in range(n):
            call = [(_tree_index(a, i) if ax is not None else a)
                    for a, ax in zip(args, axes)]
            outs.append(f(*call))
        return _tree_leaves_stack(outs)
    return inner


class custom_vjp:
    def __init__(self, fun, nondiff_argnums=()):
        self.fun = fun
        functools.update_wrapper(self, fun)

    def __call__(self, *a, **k):
        return self.fun(*a, **k)

    def defvjp(self, fwd, bwd, **_):
        self.fwd, self.bwd = fwd, bwd


def checkpoint(f=None, **_):
    if f is None:
        return lambda g: g
    return f


def grad(f, argnums=0, **_):
    """jax.grad for the small closed-form functions the reference's custom
    VJP backward passes differentiate (sum n log chi(theta) and its t-only
    variants), by central differences with two levels of Richardson
    extrapolation from steps h, h/2, h/4 (error O(h^6)) at h = 1 % of the
    entry.  The large step matters: the chi builders carry ~1e-13 of relative
    rounding noise (a Gauss-Jordan solve), which small steps would amplify;
    at this step the noise costs ~1e-8 relative and the truncation less."""
    single = isinstance(argnums, int)
    nums = (argnums,) if single else tuple(argnums)

    def g(*args):
        outs = []
        for n in nums:
            x0 = np.array(args[n], dtype=np.float64)
            flat = x0.reshape(-1)
            gflat = np.zeros_like(flat)
            for i in range(flat.size):
                def at(h, i=i):
                    xx = flat.copy()
                    xx[i] += h
                    a = list(args)
                    a[n] = _wrap(xx.reshape(x0.shape)) if x0.ndim else float(xx[0])
                    return float(np.asarray(f(*a)))
                h = 1e-2 * max(abs(flat[i]), 1e-3)
                d = [(at(h / k) - at(-h / k)) / (2 * h / k) for k in (1, 2, 4)]
                r1 = (4.0 * d[1] - d[0]) / 3.0
                r2 = (4.0 * d[2] - d[1]) / 3.0
                gflat[i] = (16.0 * r2 - r1) / 15.0
            gx = gflat.reshape(x0.shape)
            outs.append(_wrap(gx) if x0.ndim else float(gx))
        return outs[0] if single else tuple(outs)
    return g


def install():
    """Register the stand-in as ``jax`` in sys.modules."""
    jax = types.ModuleType('jax')
    jax.numpy = jnp
    jax.nn = nn
    jax.lax = lax
    jax.jit = jit
    jax.vmap = vmap
    jax.custom_vjp = custom_vjp
    jax.checkpoint = checkpoint
    jax.grad = grad
    jax.Array = np.ndarray
    cfg = types.SimpleNamespace(update=lambda *a, **k: None)
    jax.config = cfg
    jsp = types.ModuleType('jax.scipy')
    jsp_linalg = _module_proxy('jax.scipy.linalg', scipy.linalg)
    jsp_special = _module_proxy('jax.scipy.special', scipy.special,
                                {'logsumexp': logsumexp})
    jsp.linalg = jsp_linalg
    jsp.special = jsp_special
    jax.scipy = jsp
    rnd = types.ModuleType('jax.random')
    jax.random = rnd
    sys.modules.update({
        'jax': jax, 'jax.numpy': jnp, 'jax.numpy.linalg': jnp.linalg,
        'jax.nn': nn, 'jax.lax': lax, 'jax.scipy': jsp,
        'jax.scipy.linalg': jsp_linalg, 'jax.scipy.special': jsp_special,
        'jax.random': rnd,
    })
    return jax
