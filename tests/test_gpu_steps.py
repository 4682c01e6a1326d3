"""The standalone step functions rk4_step / rk2_step / euler_step
(integrators/rk4.py:62-129, rk2.py:117-180, euler.py:111-157) against the
reference's own outputs (tests/golden/steps.npz, made by running the
reference): scalar dt and per-particle dt, whose stage times come from the
mean step (rk4.py:108-129, rk2.py:163-167), at a float32 time and at Python
float times.  The float32 field is bit-exact to the reference's arithmetic,
so the steps must be too."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
from jaxtrace_gb300 import _lib as L

pytestmark = pytest.mark.gpu
F32 = np.float32


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    L.load()
    yield


@pytest.mark.parametrize("name", ["rk4", "rk2", "euler"])
@pytest.mark.parametrize("per_particle", [False, True])
def test_step_functions_match_reference(golden, name, per_particle):
    g = golden("steps")
    field = jt.StructuredTimeSeriesField(g["D"], g["st"], g["g"], g["g"], g["g"], "periodic")
    step = {"rk4": jt.rk4_step, "rk2": jt.rk2_step, "euler": jt.euler_step}[name]
    dt = g["dt_pp"] if per_particle else 0.01
    for k, t in enumerate(g["times"]):
        tf = F32(t) if k == 0 else float(t)
        out = step(g["x"], tf, dt, field)
        want = g[f"{name}_{'pp' if per_particle else 'scalar'}_{k}"]
        assert np.array_equal(out, want), (name, per_particle, k, int(np.sum(np.any(out != want, axis=1))))
