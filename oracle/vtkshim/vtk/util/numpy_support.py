"""Stand-in ``vtk.util.numpy_support`` -- TEST INFRASTRUCTURE ONLY.

``vtk_to_numpy`` follows VTK's documented shape rule: an array of one
component comes back 1-D (N,), others as (N, components)."""
import numpy as _np


def vtk_to_numpy(arr):
    a = _np.array(arr.a, copy=True)
    if a.ndim == 2 and a.shape[1] == 1:
        a = a[:, 0]
    return a
