"""``jax.numpy`` on top of NumPy, float64 by default (test infrastructure).

Only the functions the reference package and its tests call are provided.
Every array-returning function hands back a :class:`ShimArray`, which adds
JAX's out-of-place ``x.at[index].set/add/get`` API to ``numpy.ndarray``.
"""

import numpy as _np

inf, nan, pi = _np.inf, _np.nan, _np.pi
float32, float64, int32, int64 = _np.float32, _np.float64, _np.int32, _np.int64
floating, integer = _np.floating, _np.integer
finfo, iinfo, issubdtype = _np.finfo, _np.iinfo, _np.issubdtype


class _AtRef:
    def __init__(self, array, index):
        self.array, self.index = array, index

    def set(self, values):
        out = _np.array(self.array, copy=True).view(ShimArray)
        out[self.index] = values
        return out

    def add(self, values):
        out = _np.array(self.array, copy=True).view(ShimArray)
        out[self.index] = _np.asarray(out[self.index]) + values
        return out

    def get(self, mode=None, fill_value=None):
        index = self.index
        if mode == "fill" and _np.ndim(index) == 0 and not isinstance(index, (slice, tuple)):
            position = int(index)
            length = self.array.shape[0]
            if not 0 <= position < length:
                fill = _np.nan if fill_value is None else fill_value
                return _np.full(self.array.shape[1:], fill, self.array.dtype).view(ShimArray)
            return _np.asarray(self.array[position]).view(ShimArray)
        return _np.asarray(self.array[index]).view(ShimArray)


class _AtIndexer:
    def __init__(self, array):
        self.array = array

    def __getitem__(self, index):
        return _AtRef(self.array, index)


class ShimArray(_np.ndarray):
    """``numpy.ndarray`` with JAX's functional update helpers."""

    @property
    def at(self):
        return _AtIndexer(self)

    @property
    def device(self):
        return "cpu"


def _wrap(result):
    if isinstance(result, _np.ndarray):
        return result.view(ShimArray)
    return result


def _wrapped(function):
    def call(*args, **kwargs):
        return _wrap(function(*args, **kwargs))
    call.__name__ = function.__name__
    return call


def asarray(value, dtype=None):
    if dtype is None and isinstance(value, ShimArray):
        return value
    return _np.asarray(value, dtype=dtype).view(ShimArray)


array = asarray

for _name in (
    "roll", "where", "abs", "fmin", "fmax", "minimum", "maximum", "sqrt", "copysign",
    "stack", "concatenate", "sum", "mean", "min", "max", "floor", "sin", "cos", "exp",
    "zeros", "zeros_like", "ones", "ones_like", "full", "broadcast_to", "arange",
    "linspace", "meshgrid", "isfinite", "all", "any", "square", "hypot", "clip",
):
    globals()[_name] = _wrapped(getattr(_np, _name))
