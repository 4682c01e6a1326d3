"""jax.numpy as NumPy (stand-in; test infrastructure only)."""
import types as _types

import numpy as _np
from numpy import *  # noqa: F401,F403

ndarray = _np.ndarray
float32, float64, int32, int64, bool_ = _np.float32, _np.float64, _np.int32, _np.int64, _np.bool_
pi, nan, inf = _np.pi, _np.nan, _np.inf


def _det(a):
    a = _np.asarray(a)
    if a.shape[-2:] == (3, 3):
        return (a[..., 0, 0] * a[..., 1, 1] * a[..., 2, 2] +
                a[..., 0, 1] * a[..., 1, 2] * a[..., 2, 0] +
                a[..., 0, 2] * a[..., 1, 0] * a[..., 2, 1] -
                a[..., 0, 2] * a[..., 1, 1] * a[..., 2, 0] -
                a[..., 0, 0] * a[..., 1, 2] * a[..., 2, 1] -
                a[..., 0, 1] * a[..., 1, 0] * a[..., 2, 2])
    if a.shape[-2:] == (2, 2):
        return a[..., 0, 0] * a[..., 1, 1] - a[..., 0, 1] * a[..., 1, 0]
    return _np.linalg.det(a)


linalg = _types.SimpleNamespace(det=_det, norm=_np.linalg.norm, inv=_np.linalg.inv, solve=_np.linalg.solve)
