"""NumPy stand-in for the parts of ``jax`` that the reference's QG 1.5-layer
model source (mapping/models/model_qg1l/jqgm.py), its spectral Helmholtz
solvers (mapping/models/model_qgsw/helmholtz.py) and its shallow-water / QG
models (mapping/models/model_qgsw/sw.py, qg.py and their helpers) touch on
their forward paths.

Fixture generation only: ``gen_golden.py`` installs these modules in
``sys.modules`` and then loads the reference's own ``jqgm.py`` source, so that
the golden vectors are produced by the reference's lines of code executed with
NumPy float64 arithmetic in place of XLA. Nothing else imports this file.

Semantics kept from jax.numpy:
- ``x.at[idx].set(v)`` / ``.add(v)`` return a modified copy (functional update);
- ``jit`` is the identity (it only traces/compiles in jax);
- ``jnp.fft.irfft`` is NumPy's pocketfft with the same ``norm`` meaning;
- ``lax.scan`` is a Python loop, ``checkpoint`` the identity (it only changes
  what reverse mode stores), ``lax.reduce_window`` a sliding-window reduction,
  ``nn.softplus`` is log(1 + e^x) by ``logaddexp``;
- ``jnp.clip(x, a_min=...)`` accepts a missing bound, as jax's does;
- ``jnp.where(cond, size=n)`` pads / truncates the index arrays to n, and
  ``jnp.add.at(a, idx, v, inplace=False)`` returns an updated copy;
- ``vmap`` over axis 0 is a loop with stacked outputs; ``lax.dynamic_slice``
  and ``lax.dynamic_update_slice`` clamp their start indices into the operand,
  as XLA's do.
``jvp``/``vjp`` are not provided: the tangent/adjoint golden checks use finite
differences of this forward instead.
"""
import sys
import types
import functools

import numpy as np


class JArray(np.ndarray):
    """ndarray with the functional ``.at[...]`` update API of jax arrays."""

    @property
    def at(self):
        return _AtIndexer(self)


class _AtIndexer:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtUpdate(self._arr, idx)


class _AtUpdate:
    def __init__(self, arr, idx):
        self._arr = arr
        self._idx = idx

    def set(self, value):
        out = np.array(self._arr, copy=True)
        out[self._idx] = np.asarray(value)
        return out.view(JArray)

    def add(self, value):
        out = np.array(self._arr, copy=True)
        out[self._idx] += np.asarray(value)
        return out.view(JArray)


def _wrap(fn):
    @functools.wraps(fn)
    def inner(*args, **kwargs):
        out = fn(*args, **kwargs)
        if isinstance(out, np.ndarray) and not isinstance(out, JArray):
            return out.view(JArray)
        if isinstance(out, tuple):
            return tuple(o.view(JArray) if isinstance(o, np.ndarray) else o for o in out)
        return out
    return inner


class _NumpyNamespace(types.ModuleType):
    """Module whose attributes are NumPy functions returning JArray."""

    def __init__(self, name, base):
        super().__init__(name)
        self._base = base

    def __getattr__(self, name):
        attr = getattr(self._base, name)
        if callable(attr) and not isinstance(attr, type):
            return _wrap(attr)
        return attr


def _jit(fun=None, **kwargs):
    if fun is None:
        return lambda f: f
    return fun


def _scan(f, init, xs, length=None, **kwargs):
    carry, ys = init, []
    n = length if xs is None else len(xs)
    for k in range(n):
        carry, y = f(carry, None if xs is None else xs[k])
        ys.append(y)
    return carry, (None if all(y is None for y in ys) else np.stack(ys))


def _reduce_window(x, init, op, window_shape, window_strides, padding):
    """lax.reduce_window for the sums that tools.avg_pool2d asks for."""
    assert padding == "VALID"
    x = np.asarray(x)
    win = np.lib.stride_tricks.sliding_window_view(x, window_shape)
    red = init + win.sum(axis=tuple(range(x.ndim, 2 * x.ndim)))
    sl = tuple(slice(None, None, s) for s in window_strides)
    return np.ascontiguousarray(red[sl]).view(JArray)


def _clip(a, a_min=None, a_max=None, **kwargs):
    return np.clip(a, a_min, a_max).view(JArray)


def _softplus(x):
    return np.logaddexp(np.asarray(x), 0.0).view(JArray)


def _fori_loop(lower, upper, body, init):
    """jax.lax.fori_loop as the plain loop it denotes."""
    val = init
    for i in range(int(lower), int(upper)):
        val = body(i, val)
    return val


def _where(cond, x=None, y=None, size=None, fill_value=None):
    """jnp.where, with jax's ``size`` form of the one-argument call: the first
    ``size`` indices of each axis, padded with ``fill_value`` (0 by default)."""
    if x is not None or y is not None:
        return np.where(cond, x, y).view(JArray)
    idx = np.nonzero(np.asarray(cond))
    if size is None:
        return tuple(i.view(JArray) for i in idx)
    fill = 0 if fill_value is None else fill_value
    out = []
    for i in idx:
        o = np.full(size, fill, dtype=i.dtype)
        o[:min(size, i.size)] = i[:size]
        out.append(o.view(JArray))
    return tuple(out)


class _UfuncAt:
    """jnp.add / jnp.multiply with jax's functional ``.at(a, idx, v,
    inplace=False)``: the update applied to a copy."""

    def __init__(self, ufunc):
        self._u = ufunc

    def __call__(self, *args, **kwargs):
        return _wrap(self._u)(*args, **kwargs)

    def at(self, a, indices, values=None, inplace=True):
        out = np.array(np.asarray(a), copy=True)
        if values is None:
            self._u.at(out, indices)
        else:
            self._u.at(out, indices, np.asarray(values))
        return out.view(JArray)


def _unavailable(*args, **kwargs):
    raise NotImplementedError("not available in the NumPy stand-in")


def _vmap(fun, in_axes=0, out_axes=0):
    """jax.vmap over axis 0 of every argument (the form QgmWithTiles.step uses):
    a Python loop whose outputs are stacked along axis 0."""
    if in_axes != 0 or out_axes != 0:
        raise NotImplementedError("vmap stand-in: axis 0 only")

    def mapped(*args):
        n = np.shape(args[0])[0]
        outs = [fun(*(np.asarray(a)[k].view(JArray) for a in args)) for k in range(n)]
        return np.stack([np.asarray(o) for o in outs]).view(JArray)
    return mapped


def _clamped_starts(shape, starts, sizes):
    # jax.lax.dynamic_slice / dynamic_update_slice clamp every start index so
    # that the window lies inside the operand
    return [int(min(max(int(s), 0), d - z)) for s, d, z in zip(starts, shape, sizes)]


def _dynamic_slice(operand, start_indices, slice_sizes):
    x = np.asarray(operand)
    st = _clamped_starts(x.shape, start_indices, slice_sizes)
    return np.array(x[tuple(slice(a, a + z) for a, z in zip(st, slice_sizes))]).view(JArray)


def _dynamic_update_slice(operand, update, start_indices):
    x = np.array(np.asarray(operand))
    u = np.asarray(update)
    st = _clamped_starts(x.shape, start_indices, u.shape)
    x[tuple(slice(a, a + z) for a, z in zip(st, u.shape))] = u
    return x.view(JArray)


def reference_root():
    """Path of the VarDyn checkout whose files a generator loads: the first
    command-line argument, else the VARDYN_REFERENCE environment variable."""
    import os
    if len(sys.argv) > 1:
        return sys.argv[1]
    root = os.environ.get("VARDYN_REFERENCE")
    if not root:
        raise SystemExit("usage: python %s <VarDyn checkout>  (or set VARDYN_REFERENCE)" % sys.argv[0])
    return root


def install(enable_x64=True):
    """Register fake ``jax``, ``matplotlib`` and ``src.config`` modules."""
    jax = types.ModuleType("jax")
    jnp = _NumpyNamespace("jax.numpy", np)
    jnp.fft = _NumpyNamespace("jax.numpy.fft", np.fft)
    jnp.linalg = _NumpyNamespace("jax.numpy.linalg", np.linalg)
    jnp.clip = _clip
    jnp.where = _where
    jnp.add = _UfuncAt(np.add)
    jax.numpy = jnp
    jax.jit = _jit
    jax.checkpoint = lambda f, **kw: f
    nn = types.ModuleType("jax.nn")
    nn.softplus = _softplus
    jax.nn = nn
    jax.jvp = _unavailable
    jax.vjp = _unavailable
    jax.vmap = _vmap
    cfg = types.SimpleNamespace(update=lambda *a, **k: None)
    jax.config = cfg
    lax = types.ModuleType("jax.lax")
    lax.fori_loop = _fori_loop
    lax.dynamic_slice = _dynamic_slice
    lax.dynamic_update_slice = _dynamic_update_slice
    lax.scan = _scan
    lax.reduce_window = _reduce_window
    lax.add = np.add
    jax.lax = lax
    jsp = types.ModuleType("jax.scipy")
    jsp_sparse = types.ModuleType("jax.scipy.sparse")
    jsp_linalg = types.ModuleType("jax.scipy.sparse.linalg")
    jsp_linalg.cg = _unavailable
    jsp.sparse = jsp_sparse
    jsp_sparse.linalg = jsp_linalg
    jax.scipy = jsp

    mpl = types.ModuleType("matplotlib")
    pylab = types.ModuleType("matplotlib.pylab")
    pyplot = types.ModuleType("matplotlib.pyplot")
    mpl.pylab = pylab
    mpl.pyplot = pyplot

    src = types.ModuleType("src")
    src_config = types.ModuleType("src.config")
    src_config.USE_FLOAT64 = bool(enable_x64)
    src.config = src_config

    sys.modules.update({
        "jax": jax, "jax.numpy": jnp, "jax.numpy.fft": jnp.fft,
        "jax.lax": lax, "jax.nn": nn, "jax.numpy.linalg": jnp.linalg, "jax.scipy": jsp, "jax.scipy.sparse": jsp_sparse,
        "jax.scipy.sparse.linalg": jsp_linalg,
        "matplotlib": mpl, "matplotlib.pylab": pylab, "matplotlib.pyplot": pyplot,
        "src": src, "src.config": src_config,
    })
