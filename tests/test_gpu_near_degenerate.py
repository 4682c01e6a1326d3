"""Near-degenerate tetrahedra: in the compensated arithmetic the barycentric
weights of a tetrahedron whose |det| is below 1e-2 of the product of its
edge lengths are solved again in float64 (the float32 solve still decides
which tetrahedron holds the query, as in the reference).  On a rotated
sliver with a linear velocity field, P1 interpolation is then exact to
float32 rounding, where the float32 solve loses digits to cancellation."""
import ctypes as C

import numpy as np
import pytest

import jaxtrace_gb300 as jt
from jaxtrace_gb300 import _lib as L

pytestmark = pytest.mark.gpu
F32 = np.float32


def _sample(field, q, arith):
    import torch
    field._device()
    qd = torch.from_numpy(np.ascontiguousarray(q, dtype=F32)).cuda()
    out = torch.empty_like(qd)
    blend = L.Blend.from_buffer_copy(field.blend_at(0.5).tobytes())
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    L.check(L.load().jt_field_sample(C.byref(field._cfield), C.byref(blend), arith, L.ptr(qd), L.ptr(out),
                                     qd.shape[0], L.ptr(status), L.stream_ptr()))
    return out.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("kind", ["octree", "hash_grid"])
def test_sliver_weights_are_solved_in_float64(kind):
    rng = np.random.default_rng(11)
    base = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.3, 0.3, 1e-4]])
    R, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    P = (base @ R.T + np.array([0.5, 0.2, 0.1])).astype(F32)
    T4 = np.array([[0, 1, 2, 3]], np.int32)
    A, c0 = rng.normal(size=(3, 3)), rng.normal(size=3)
    vals = (P.astype(np.float64) @ A.T + c0).astype(F32)
    data, times = np.stack([vals, vals]), np.array([0.0, 1.0], F32)
    if kind == "octree":
        f = jt.OctreeFEMTimeSeriesFieldOptimized(data, times, P, T4)
    else:
        f = jt.FEMTimeSeriesField(data, times, P, T4, fem_grid_resolution=2)
    lam = rng.dirichlet(np.full(4, 5.0), size=400)
    lam = lam[lam.min(axis=1) > 0.05]
    Q = (lam @ P.astype(np.float64)).astype(F32)
    # truth: float64 weights from the stored float32 geometry, float64 P1 sum
    v0 = P[0].astype(np.float64)
    D = np.stack([(P[k] - P[0]).astype(F32).astype(np.float64) for k in (1, 2, 3)], axis=1)
    w = np.linalg.solve(D, (Q.astype(np.float64) - v0).T).T
    truth = (1 - w.sum(axis=1))[:, None] * vals[0] + w @ vals[1:].astype(np.float64)
    err_exact = np.abs(_sample(f, Q, L.JT_ARITH_EXACT) - truth).max()
    err_comp = np.abs(_sample(f, Q, L.JT_ARITH_COMPENSATED) - truth).max()
    assert f.n_near_degenerate == 1
    scale = np.abs(vals).max()
    assert err_comp < 1e-6 * scale * 10
    assert err_exact > 10 * err_comp          # the float32 solve loses digits here
