"""A NumPy stand-in for the small part of the jax API that the AeroJAX
projection-step source files use.  Test infrastructure only: it lets
``make_golden.py`` execute the reference's *own* Python files (which cannot
run here because jax is not installed) in float64 and record their outputs as
golden fixtures.

Semantics restated from the public JAX documentation:
  * ``jax.jit`` returns the function unchanged (tracing does not change the
    arithmetic of these stencil functions);
  * ``x.at[idx].set(y)`` / ``.add(y)`` / ``.get()`` return a modified copy /
    the indexed value (immutable update);
  * ``jax.lax.scan(f, init, xs)`` loops over the leading axis of ``xs``;
  * ``jax.lax.cond(p, t, f, *ops)`` evaluates the selected branch;
  * ``jax.nn.sigmoid`` is the logistic function;
  * with x64 enabled, ``float`` and the default dtype are float64.
"""
from __future__ import annotations

import sys
import types

import numpy as np

DEFAULT_DTYPE = np.float64


class _AtIndexer:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtRef(self._arr, idx)


class _AtRef:
    def __init__(self, arr, idx):
        self._arr, self._idx = arr, idx

    def set(self, val):
        out = np.array(self._arr, copy=True).view(JArr)
        out[self._idx] = np.asarray(val)
        return out

    def add(self, val):
        out = np.array(self._arr, copy=True).view(JArr)
        out[self._idx] += np.asarray(val)
        return out

    def get(self):
        return _wrap(np.asarray(self._arr)[self._idx])


class JArr(np.ndarray):
    """ndarray with JAX's functional ``.at`` update property."""

    @property
    def at(self):
        return _AtIndexer(self)


def _wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, JArr):
        return x.view(JArr)
    if isinstance(x, tuple):
        return tuple(_wrap(e) for e in x)
    if isinstance(x, list):
        return [_wrap(e) for e in x]
    return x


def _wrapped(fn):
    def inner(*a, **k):
        return _wrap(fn(*a, **k))
    inner.__name__ = getattr(fn, "__name__", "fn")
    return inner


# ---------------------------------------------------------------- jax.numpy
jnp = types.ModuleType("jax.numpy")


def _creation(fn):
    def inner(shape, dtype=None, **k):
        return _wrap(fn(shape, dtype=DEFAULT_DTYPE if dtype is None else dtype, **k))
    return inner


jnp.zeros = _creation(np.zeros)
jnp.ones = _creation(np.ones)


def _full(shape, fill_value, dtype=None):
    return _wrap(np.full(shape, fill_value, dtype=DEFAULT_DTYPE if dtype is None else dtype))


jnp.full = _full


def _array(x, dtype=None, **k):
    a = np.array(x, dtype=dtype)
    if dtype is None and a.dtype.kind == "f":
        a = a.astype(DEFAULT_DTYPE)
    return _wrap(a)


jnp.array = _array
jnp.asarray = _array
jnp.ndarray = np.ndarray
jnp.pi = np.pi
jnp.float32 = np.float32
jnp.float64 = np.float64
jnp.int32 = np.int32
jnp.linalg = types.SimpleNamespace(norm=_wrapped(np.linalg.norm))


def _jnp_getattr(name):
    fn = getattr(np, name)
    if callable(fn):
        return _wrapped(fn)
    return fn


jnp.__getattr__ = _jnp_getattr

# ---------------------------------------------------------------- jax.lax
lax = types.ModuleType("jax.lax")


def scan(f, init, xs=None, length=None):
    carry = init
    ys = []
    n = len(xs) if xs is not None else length
    for k in range(n):
        carry, y = f(carry, None if xs is None else xs[k])
        ys.append(y)
    if ys and ys[0] is not None:
        return carry, _wrap(np.stack([np.asarray(y) for y in ys]))
    return carry, None


def cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if bool(np.asarray(pred)) else false_fun(*operands)


lax.scan = scan
lax.cond = cond

# ---------------------------------------------------------------- jax.nn
nn = types.ModuleType("jax.nn")


def sigmoid(x):
    x = np.asarray(x, dtype=np.result_type(np.asarray(x).dtype, DEFAULT_DTYPE))
    out = np.empty_like(x)
    pos = x >= 0
    out[pos] = 1.0 / (1.0 + np.exp(-x[pos]))
    ex = np.exp(x[~pos])
    out[~pos] = ex / (1.0 + ex)
    return _wrap(out)


nn.sigmoid = sigmoid
nn.relu = _wrapped(lambda x: np.maximum(x, 0))

# ---------------------------------------------------------------- jax
jax = types.ModuleType("jax")


def _to_jarr(x):
    if isinstance(x, np.ndarray) and not isinstance(x, JArr):
        return x.view(JArr)
    if isinstance(x, float):
        return np.float64(x)     # traced scalars divide like arrays (0/0 -> nan)
    return x


def jit(fun=None, **kw):
    """Arguments become arrays with ``.at`` (as jax arrays would); the
    function body runs unchanged."""
    if fun is None:
        return lambda f: jit(f, **kw)

    def call(*a, **k):
        with np.errstate(divide="ignore", invalid="ignore"):
            return fun(*[_to_jarr(x) for x in a], **{n: _to_jarr(x) for n, x in k.items()})
    call.__name__ = getattr(fun, "__name__", "jitted")
    call.__wrapped__ = fun
    return call


jax.jit = jit
jax.numpy = jnp
jax.lax = lax
jax.nn = nn
jax.tree_util = types.SimpleNamespace(register_dataclass=lambda c: c,
                                      tree_map=lambda f, *t: f(*t))
jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
jax.clear_caches = lambda: None
_scipy = types.ModuleType("jax.scipy")
_ndimage = types.ModuleType("jax.scipy.ndimage")
_ndimage.map_coordinates = None
_scipy.ndimage = _ndimage
jax.scipy = _scipy
jnp.lax = lax


def install():
    """Register the stand-in modules under the ``jax`` names."""
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jnp
    sys.modules["jax.lax"] = lax
    sys.modules["jax.nn"] = nn
    sys.modules["jax.scipy"] = _scipy
    sys.modules["jax.scipy.ndimage"] = _ndimage
