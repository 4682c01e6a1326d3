"""NumPy stand-in for the subset of ``jax`` that JAXTrace's tracking modules
use -- TEST INFRASTRUCTURE ONLY (lets the reference's octree modules, which
import jax unconditionally, run in a container without JAX when golden
fixtures are regenerated).

jit is the identity, vmap a Python loop, lax control flow plain Python and
jax.numpy is NumPy except ``linalg.det`` of 3x3 matrices, which uses the
closed-form expansion JAX applies to 3x3 inputs (six triple products summed
left to right) instead of NumPy's LU/log-det route.
"""
import numpy as _np

from . import lax, numpy  # noqa: F401

__version__ = "0.0+numpy-stand-in"
Array = _np.ndarray


def jit(fn=None, **kwargs):
    if fn is None:
        return lambda f: f
    return fn


def vmap(fn, in_axes=0, out_axes=0):
    def _mapped(*args):
        n = len(args[0])
        res = [fn(*[a[i] for a in args]) for i in range(n)]
        if isinstance(res[0], tuple):
            return tuple(_np.stack([_np.asarray(r[k]) for r in res]) for k in range(len(res[0])))
        return _np.stack([_np.asarray(r) for r in res])
    return _mapped


def device_put(x, *args, **kwargs):
    return _np.asarray(x)


def devices(kind=None):
    return []
