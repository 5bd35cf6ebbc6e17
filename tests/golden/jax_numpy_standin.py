"""A numpy stand-in for the parts of jax and flax that larnd-sim-jax's LUT
simulate path uses, so that the reference's own source files can run in a
process without JAX and produce golden vectors (make_lut_golden.py).

Test infrastructure only: nothing in the package imports it.  It encodes
JAX's documented semantics with 64-bit types disabled (the reference never
enables them):

* every array is 32-bit (unless installed with x64=True, JAX's
  jax_enable_x64): float64 / int64 results, numpy float64 inputs and
  ``astype(int)`` / ``astype(float)`` narrow to float32 / int32, while
  Python scalars stay weakly typed (numpy 2 follows the same promotion rule
  for them, NEP 50), except that an integer array met by a Python float,
  or divided, is converted to float32 first, as JAX does, instead of being
  computed in float64;
* gathers (``x[idx]`` with integer arrays) wrap negative indices once and
  clamp the rest into range;
* ``take`` wraps negative indices once and fills out-of-range positions
  (NaN for floats), its default mode;
* scatters (``x.at[idx].set/add/...``) wrap negative indices once and drop
  out-of-range updates; ``jax.ops.segment_sum`` drops segment ids outside
  ``[0, num_segments)``;
* ``jnp.linspace`` evaluates ``start*(1 - i/div) + stop*(i/div)`` in float32
  with ``stop`` appended exactly;
* ``jit``, ``checkpoint``, ``stop_gradient`` and the profiler annotations
  are identities, ``vmap`` and ``lax.scan`` are Python loops, and
  ``jax.random`` draws from numpy generators (not JAX's threefry stream, so
  only runs whose noise amplitudes are zero are reproducible).

Element-wise float32 arithmetic is IEEE in both; transcendental functions
(erf from scipy, exp and log from numpy) and the order of reductions
(cumsum, scatter-add) can differ from XLA's by a few ulp.
"""

from __future__ import annotations

import dataclasses
import sys
import types

import numpy as np
import scipy.special
import scipy.stats

_NARROW = {np.dtype(np.float64): np.dtype(np.float32), np.dtype(np.int64): np.dtype(np.int32),
           np.dtype(np.uint64): np.dtype(np.uint32), np.dtype(np.complex128): np.dtype(np.complex64)}


_X64 = [False]      # install(x64=True): JAX with jax_enable_x64, nothing narrowed


def _narrow_dtype(dt):
    dt = np.dtype(dt)
    return dt if _X64[0] else _NARROW.get(dt, dt)


class JArr(np.ndarray):
    """An immutable-by-convention 32-bit array with JAX's indexing rules."""

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        if kwargs.get("out") is not None:
            raise TypeError("JAX arrays are immutable: no out= arguments")
        args = [_plain(_x32(x)) for x in inputs]
        res = getattr(ufunc, method)(*args, **kwargs)
        if not _X64[0] and any(np.asarray(r).dtype == np.float64 for r in (res if isinstance(res, tuple) else (res,))):
            # numpy promotes an int32 operand with a Python float (or a true
            # division of integers) to float64; JAX converts the integer
            # operand to float32 and computes in float32
            args = [a.astype(np.float32) if isinstance(a, np.ndarray) and a.dtype.kind in "iub" else a
                    for a in args]
            res = getattr(ufunc, method)(*args, **kwargs)
        return _x32(res)

    def __array_wrap__(self, obj, context=None, return_scalar=False):
        return _x32(np.asarray(obj))

    def __getitem__(self, idx):
        idx, _ = _normalise_index(self.shape, idx, clamp=True)
        return _x32(_plain(self)[idx])

    def __setitem__(self, idx, value):
        raise TypeError("JAX arrays are immutable: use .at[...]")

    def astype(self, dtype, *args, **kwargs):
        return _x32(np.asarray(_plain(self)).astype(_narrow_dtype(dtype)))

    def take(self, indices, axis=None, out=None, mode=None, unique_indices=False, indices_are_sorted=False,
             fill_value=None):
        return take(self, indices, axis=axis, mode=mode, fill_value=fill_value)

    def argmax(self, *args, **kwargs):
        return _x32(_plain(self).argmax(*args, **kwargs))

    def argmin(self, *args, **kwargs):
        return _x32(_plain(self).argmin(*args, **kwargs))

    def argsort(self, *args, **kwargs):
        return _x32(_plain(self).argsort(*args, **kwargs))

    def nonzero(self):
        return tuple(_x32(r) for r in _plain(self).nonzero())

    @property
    def at(self):
        return _AtIndexer(self)


def _plain(x):
    return x.view(np.ndarray) if isinstance(x, np.ndarray) and type(x) is not np.ndarray else x


def _x32(v):
    """Arrays and numpy scalars into the 32-bit world; tuples and lists
    element by element; Python scalars and other objects unchanged."""
    if isinstance(v, (np.ndarray, np.generic)):
        a = np.asarray(v)
        nd = _narrow_dtype(a.dtype)
        if nd != a.dtype:
            a = a.astype(nd)
        return a.view(JArr)
    if isinstance(v, tuple):
        return tuple(_x32(x) for x in v)
    if isinstance(v, list):
        return [_x32(x) for x in v]
    return v


def _arg(v):
    """A function argument for numpy: 32-bit, plain ndarray."""
    if isinstance(v, (np.ndarray, np.generic)):
        return _plain(_x32(v))
    if isinstance(v, tuple):
        return tuple(_arg(x) for x in v)
    if isinstance(v, list):
        return [_arg(x) for x in v]
    return v


def _consumes(c):
    if c is None or c is Ellipsis:
        return 0
    if isinstance(c, np.ndarray) and c.dtype == bool:
        return c.ndim
    return 1


def _normalise_index(shape, idx, clamp):
    """The index with JAX's integer-array rules applied: negative entries
    wrapped once; then clamped (gather) or left for the caller to drop
    (scatter).  Returns the index and, per component, the size of the axis
    an integer array indexes (None for the other components)."""
    if not isinstance(idx, tuple):
        idx = (idx,)
    comps = []
    for c in idx:
        if isinstance(c, list):
            c = np.asarray(c)
        if isinstance(c, np.ndarray):
            c = _plain(_x32(c))
        elif isinstance(c, np.integer):
            c = int(c)
        elif isinstance(c, np.bool_):
            c = np.asarray(c)
        comps.append(c)
    n_used = sum(_consumes(c) for c in comps)
    axis, out, sizes = 0, [], []
    for c in comps:
        size = None
        if c is Ellipsis:
            axis += len(shape) - n_used
        elif c is None:
            pass
        elif isinstance(c, np.ndarray) and c.dtype.kind in "iu":
            size = shape[axis]
            c = np.where(c < 0, c + size, c)
            if clamp:
                c = np.clip(c, 0, size - 1)
            axis += 1
        elif isinstance(c, np.ndarray) and c.dtype == bool:
            axis += c.ndim
        elif isinstance(c, np.ndarray):
            raise TypeError(f"index arrays must be integer or boolean, got {c.dtype}")
        else:
            axis += 1
        out.append(c)
        sizes.append(size)
    return tuple(out), sizes


class _AtIndexer:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtRef(self._arr, idx)


class _AtRef:
    """``x.at[idx]``: functional updates that drop out-of-range positions."""

    def __init__(self, arr, idx):
        self._arr, self._idx = arr, idx

    def get(self, mode=None, fill_value=None, **kwargs):
        if mode not in (None, "clip", "promise_in_bounds"):
            raise NotImplementedError(f".at[].get(mode={mode!r})")
        return self._arr[self._idx]

    def _scatter(self, values, op):
        out = np.array(_plain(self._arr), copy=True)
        idx, sizes = _normalise_index(out.shape, self._idx, clamp=False)
        vals = np.asarray(_arg(values)).astype(out.dtype)
        adv = [k for k, s in enumerate(sizes) if s is not None]
        if adv:
            valid = np.ones(np.broadcast_shapes(*[idx[k].shape for k in adv]), bool)
            for k in adv:
                valid &= (idx[k] >= 0) & (idx[k] < sizes[k])
            if not valid.all():
                if len(idx) != 1:
                    raise NotImplementedError("out-of-range scatter with a multi-component index")
                keep = idx[0][valid]
                vals = np.broadcast_to(vals, idx[0].shape)[valid] if vals.ndim else vals
                idx = (keep,)
        if op is None:
            out[idx] = vals
        else:
            op.at(out, idx, vals)
        return out.view(JArr)

    def set(self, values, **kwargs):
        return self._scatter(values, None)

    def add(self, values, **kwargs):
        return self._scatter(values, np.add)

    def subtract(self, values, **kwargs):
        return self._scatter(values, np.subtract)

    def multiply(self, values, **kwargs):
        return self._scatter(values, np.multiply)

    def min(self, values, **kwargs):
        return self._scatter(values, np.minimum)

    def max(self, values, **kwargs):
        return self._scatter(values, np.maximum)


def take(a, indices, axis=None, out=None, mode=None, unique_indices=False, indices_are_sorted=False,
         fill_value=None):
    """jnp.take: negative indices wrapped once, then 'fill' (default: NaN for
    floats, the most negative value for signed integers), 'clip' or 'wrap'."""
    arr = _plain(_x32(np.asarray(a)))
    ind = _plain(_x32(np.asarray(indices)))
    if axis is None:
        arr, axis = arr.ravel(), 0
    n = arr.shape[axis]
    if mode in (None, "fill"):
        ind = np.where(ind < 0, ind + n, ind)
        valid = (ind >= 0) & (ind < n)
        res = np.take(arr, np.where(valid, ind, 0), axis=axis)
        if not valid.all():
            if fill_value is None:
                fill_value = np.nan if arr.dtype.kind in "fc" else (
                    np.iinfo(arr.dtype).min if arr.dtype.kind == "i" else np.iinfo(arr.dtype).max)
            ax = axis % arr.ndim
            m = valid.reshape((1,) * ax + valid.shape + (1,) * (arr.ndim - ax - 1))
            res = np.where(m, res, np.asarray(fill_value).astype(arr.dtype))
    elif mode in ("clip", "wrap"):
        res = np.take(arr, ind, axis=axis, mode=mode)
    else:
        raise NotImplementedError(f"take(mode={mode!r})")
    return _x32(res)


# ---------------------------------------------------------------- jax.numpy

def _wrap_np(fn):
    if isinstance(fn, np.ufunc):
        def call_ufunc(*args, **kwargs):
            # dispatch through JArr.__array_ufunc__ (JAX's promotion)
            return _x32(fn(*[_x32(a) if isinstance(a, (np.ndarray, np.generic)) else a for a in args], **kwargs))
        call_ufunc.__name__ = fn.__name__
        return call_ufunc

    def call(*args, **kwargs):
        kwargs = {k: (_narrow_dtype(v) if k == "dtype" and v is not None else _arg(v)) for k, v in kwargs.items()}
        return _x32(fn(*[_arg(a) for a in args], **kwargs))
    call.__name__ = getattr(fn, "__name__", "jnp_function")
    return call


def linspace(start, stop, num=50, endpoint=True, retstep=False, dtype=None, axis=0):
    if not endpoint or retstep or axis != 0:
        raise NotImplementedError("linspace with endpoint=False, retstep or axis")
    ft = np.float64 if _X64[0] else np.float32
    s, e = ft(start), ft(stop)
    if num == 1:
        return _x32(np.array([s], ft))
    div = num - 1
    step = (np.arange(div, dtype=ft) / ft(div)).astype(ft)
    body = (s * (ft(1) - step) + e * step).astype(ft)
    return _x32(np.concatenate([body, np.array([e], ft)]))


def where(condition, x=None, y=None, *, size=None, fill_value=None):
    if x is None and y is None:
        rows = np.nonzero(_arg(np.asarray(condition)))
        if size is not None:
            fv = 0 if fill_value is None else fill_value
            rows = tuple(np.concatenate([r[:size], np.full(max(size - r.shape[0], 0), fv, r.dtype)]) for r in rows)
        return tuple(_x32(r) for r in rows)
    return _x32(np.where(_arg(condition), _arg(x), _arg(y)))


def searchsorted(a, v, side="left", sorter=None, *, method=None):
    return _x32(np.searchsorted(_arg(a), _arg(v), side=side, sorter=sorter))


def unique(ar, return_index=False, return_inverse=False, return_counts=False, axis=None, *, size=None,
           fill_value=None, **kwargs):
    if size is not None:
        raise NotImplementedError("unique(size=...)")
    return _x32(np.unique(_arg(ar), return_index=return_index, return_inverse=return_inverse,
                          return_counts=return_counts, axis=axis))


class _Grid:
    def __init__(self, grid):
        self._grid = grid

    def __getitem__(self, key):
        return _x32(self._grid[key])


class _NumpyNamespace(types.ModuleType):
    """jax.numpy: numpy's functions with 32-bit results, the overrides
    above, and numpy's scalar types and constants as they are."""

    def __getattr__(self, name):
        obj = getattr(np, name)
        if isinstance(obj, type) or not callable(obj):
            return obj
        return _wrap_np(obj)


def _make_jnp():
    m = _NumpyNamespace("jax.numpy")
    m.ndarray = np.ndarray
    m.newaxis = None
    m.take = take
    m.linspace = linspace
    m.where = where
    m.searchsorted = searchsorted
    m.unique = unique
    m.mgrid = _Grid(np.mgrid)
    m.ogrid = _Grid(np.ogrid)
    m.asarray = _wrap_np(np.asarray)
    m.array = _wrap_np(np.array)
    return m


# ---------------------------------------------------------------- jax.lax, jax.random, jax.nn, jax.ops

def _stack(outs):
    first = outs[0]
    if isinstance(first, tuple):
        return tuple(_stack([o[i] for o in outs]) for i in range(len(first)))
    if first is None:
        return None
    return _x32(np.stack([_arg(np.asarray(o)) for o in outs]))


def scan(f, init, xs=None, length=None, reverse=False, unroll=1, **kwargs):
    if reverse:
        raise NotImplementedError("scan(reverse=True)")
    n = length if xs is None else len(xs[0] if isinstance(xs, tuple) else xs)
    carry, ys = init, []
    for i in range(n):
        x = None if xs is None else (tuple(v[i] for v in xs) if isinstance(xs, tuple) else xs[i])
        carry, y = f(carry, x)
        ys.append(y)
    return carry, (_stack(ys) if ys else None)


def cummax(operand, axis=0, reverse=False):
    a = _arg(np.asarray(operand))
    if reverse:
        return _x32(np.flip(np.maximum.accumulate(np.flip(a, axis), axis=axis), axis))
    return _x32(np.maximum.accumulate(a, axis=axis))


def associative_scan(fn, elems, reverse=False, axis=0):
    """Inclusive scan of a binary associative ``fn`` along ``axis``,
    evaluated left to right (the result of an associative fn does not
    depend on the grouping)."""
    if reverse:
        raise NotImplementedError("associative_scan(reverse=True)")
    a = np.moveaxis(_arg(np.asarray(elems)), axis, 0)
    if a.shape[0] == 0:
        return _x32(np.moveaxis(a, 0, axis))
    out = [a[0]]
    for i in range(1, a.shape[0]):
        out.append(_arg(np.asarray(fn(out[-1], a[i]))))
    return _x32(np.moveaxis(np.stack(out), 0, axis))


def top_k(operand, k):
    a = _arg(np.asarray(operand))
    idx = np.argsort(-a, axis=-1, kind="stable")[..., :k]
    return _x32(np.take_along_axis(a, idx, axis=-1)), _x32(idx)


def cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if bool(pred) else false_fun(*operands)


def fori_loop(lower, upper, body_fun, init_val, **kwargs):
    val = init_val
    for i in range(int(lower), int(upper)):
        val = body_fun(i, val)
    return val


def _identity(x):
    return x


def jit(fun=None, **kwargs):
    return fun if fun is not None else _identity


def vmap(fun, in_axes=0, out_axes=0, **kwargs):
    if out_axes != 0:
        raise NotImplementedError("vmap(out_axes != 0)")

    def mapped(*args):
        axes = tuple(in_axes) if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = next(np.shape(a)[ax] for a, ax in zip(args, axes) if ax is not None)
        outs = [fun(*[a if ax is None else _x32(np.take(_arg(np.asarray(a)), i, axis=ax)) for a, ax in zip(args, axes)])
                for i in range(n)]
        return _stack(outs)
    return mapped


def _rng(key):
    return np.random.default_rng(np.asarray(key, np.uint32).ravel().tolist())


def prng_key(seed):
    return np.array([0, int(seed) & 0xFFFFFFFF], dtype=np.uint32)


def split(key, num=2):
    return _rng(key).integers(0, 2 ** 32, size=(num, 2), dtype=np.uint32)


def normal(key, shape=(), dtype=np.float32):
    return _x32(_rng(key).standard_normal(shape).astype(np.float32))


def uniform(key, shape=(), dtype=np.float32, minval=0.0, maxval=1.0):
    return _x32(_rng(key).uniform(minval, maxval, shape).astype(np.float32))


def segment_sum(data, segment_ids, num_segments=None, indices_are_sorted=False, unique_indices=False,
                bucket_size=None, mode=None):
    d = _arg(np.asarray(data))
    ids = _arg(np.asarray(segment_ids))
    if num_segments is None:
        num_segments = int(ids.max()) + 1
    out = np.zeros((num_segments,) + d.shape[ids.ndim:], d.dtype)
    keep = (ids >= 0) & (ids < num_segments)
    np.add.at(out, ids[keep], d[keep])
    return _x32(out)


class _Norm:
    @staticmethod
    def pdf(x, loc=0, scale=1):
        return _x32(scipy.stats.norm.pdf(_arg(x), loc=_arg(loc), scale=_arg(scale)))

    @staticmethod
    def cdf(x, loc=0, scale=1):
        return _x32(scipy.stats.norm.cdf(_arg(x), loc=_arg(loc), scale=_arg(scale)))

    @staticmethod
    def logpdf(x, loc=0, scale=1):
        return _x32(scipy.stats.norm.logpdf(_arg(x), loc=_arg(loc), scale=_arg(scale)))


class _SpecialNamespace(types.ModuleType):
    def __getattr__(self, name):
        return _wrap_np(getattr(scipy.special, name))


# ---------------------------------------------------------------- flax.struct, yaml, h5py

def struct_field(pytree_node=True, **kwargs):
    return dataclasses.field(metadata={"pytree_node": pytree_node}, **kwargs)


def struct_dataclass(clz=None, **kwargs):
    def make(c):
        dc = dataclasses.dataclass(frozen=True, **kwargs)(c)
        dc.replace = lambda self, **updates: dataclasses.replace(self, **updates)
        return dc
    return make(clz) if clz is not None else make


def _module(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    return m


def install(yaml_loads, x64=False):
    """Register jax, flax, yaml (parsed with ``yaml_loads(text)``) and an
    empty h5py in sys.modules.  Call before importing the reference.
    ``x64``: JAX's semantics with jax_enable_x64 (64-bit types kept, float64
    linspace); a float32 input array then still computes in float32."""
    _X64[0] = bool(x64)
    jnp = _make_jnp()
    lax = _module("jax.lax", scan=scan, cummax=cummax, top_k=top_k, cond=cond, fori_loop=fori_loop,
                  stop_gradient=_identity, associative_scan=associative_scan)
    random = _module("jax.random", key=prng_key, PRNGKey=prng_key, split=split, normal=normal, uniform=uniform)
    special = _SpecialNamespace("jax.scipy.special")
    stats = _module("jax.scipy.stats", norm=_Norm())
    scipy_mod = _module("jax.scipy", special=special, stats=stats)
    nn = _module("jax.nn", sigmoid=_wrap_np(scipy.special.expit), softplus=lambda x: _x32(np.logaddexp(0, _arg(x))),
                 logsumexp=_wrap_np(scipy.special.logsumexp), softmax=_wrap_np(scipy.special.softmax))
    ops = _module("jax.ops", segment_sum=segment_sum)
    profiler = _module("jax.profiler", annotate_function=lambda f=None, **k: f if f is not None else _identity)
    debug = _module("jax.debug", print=lambda *a, **k: None)
    experimental = _module("jax.experimental")
    tree_util = _module("jax.tree_util")
    jax = _module("jax", numpy=jnp, lax=lax, random=random, scipy=scipy_mod, nn=nn, ops=ops, profiler=profiler,
                  debug=debug, experimental=experimental, tree_util=tree_util, jit=jit, vmap=vmap,
                  checkpoint=lambda f=None, **k: f if f is not None else _identity, Array=np.ndarray,
                  named_scope=lambda name: _identity)
    struct = _module("flax.struct", field=struct_field, dataclass=struct_dataclass)
    flax = _module("flax", struct=struct)

    class _Loader:
        pass

    yaml = _module("yaml", load=lambda stream, Loader=None: yaml_loads(stream.read()), safe_load=
                   lambda stream: yaml_loads(stream.read()), FullLoader=_Loader, SafeLoader=_Loader)
    for name, mod in {"jax": jax, "jax.numpy": jnp, "jax.lax": lax, "jax.random": random, "jax.scipy": scipy_mod,
                      "jax.scipy.special": special, "jax.scipy.stats": stats, "jax.nn": nn, "jax.ops": ops,
                      "jax.profiler": profiler, "jax.debug": debug, "jax.experimental": experimental,
                      "jax.tree_util": tree_util, "flax": flax, "flax.struct": struct, "yaml": yaml,
                      "h5py": _module("h5py")}.items():
        sys.modules[name] = mod
