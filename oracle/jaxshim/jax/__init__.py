"""A NumPy-backed stand-in for the small part of JAX that JathenAX uses.

Test infrastructure only. It lets the unmodified reference package
(``jathenax/*.py``) run on a machine without jax/jaxlib, in float64 ("x64")
mode, so that its own tests can be run and golden vectors generated from it.
``jit`` is the identity, ``lax`` control flow is ordinary Python control flow,
and arrays are ``numpy.ndarray`` subclasses that add JAX's functional
``.at[...]`` update syntax.

Nothing in the shipped package imports this module.
"""

from functools import partial as _partial

import numpy as _np

from . import numpy  # noqa: F401  (exposes jax.numpy)
from . import lax  # noqa: F401
from .numpy import ShimArray as _ShimArray


class _Config:
    """``jax.config``: settings are accepted and ignored (x64 is always on)."""

    def update(self, name, value):
        self.__dict__[name] = value


config = _Config()


def jit(fun=None, **options):
    """Identity transform; keyword options such as ``static_argnames`` are ignored."""
    if fun is None:
        return _partial(jit, **options)
    return fun


def _tree_map(function, tree):
    if isinstance(tree, dict):
        return {key: _tree_map(function, value) for key, value in tree.items()}
    if isinstance(tree, (tuple, list)):
        return type(tree)(_tree_map(function, value) for value in tree)
    if tree is None:
        return None
    return function(tree)


def device_get(tree):
    """Return plain NumPy arrays (scalars stay NumPy scalars)."""
    def get(leaf):
        if isinstance(leaf, _np.ndarray):
            return _np.asarray(leaf).view(_np.ndarray)
        return leaf
    return _tree_map(get, tree)


def device_put(tree, device=None):
    def put(leaf):
        if isinstance(leaf, (_np.ndarray, _np.generic, float, int, bool)):
            return _np.asarray(leaf).view(_ShimArray)
        return leaf
    return _tree_map(put, tree)


def devices():
    return ["cpu"]
