"""The CPU oracle against golden vectors produced by running the reference
(tests/golden/make_golden.py).  Float32 results are compared bit for bit."""
import numpy as np
import pytest

import oracle

F32 = np.float32


def same(a, b):
    """Bitwise equality with NaN == NaN."""
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("ex", ["constant", "linear", "zero", "nan"])
def test_time_blend(golden, ex):
    g = golden("time_blend")
    spec = oracle.NearestSpec(g["data"], g["times"], np.zeros((g["data"].shape[1], 3), F32), extrapolation=ex)
    for i, t in enumerate(g["tq"]):
        assert same(oracle.blend_nodes(spec, float(t)), g[f"out_{ex}"][i]), (ex, t)


@pytest.mark.parametrize("mode", ["clamp", "zero", "nan", "periodic"])
def test_structured_sampler(golden, mode):
    g = golden("structured")
    V = g[f"{mode}_V"]
    spec = oracle.GridSpec(V[None], np.zeros(1, F32), g[f"{mode}_gx"], g[f"{mode}_gy"], g[f"{mode}_gz"], mode)
    out, _ = oracle.sample(spec, g[f"{mode}_q"], 0.0)
    assert same(out, g[f"{mode}_out"])


CASES = {
    "periodic": dict(kinds=("periodic",) * 3),
    "reflective": dict(kinds=("reflective",) * 3),
    "clamping": dict(kinds=("clamping",) * 3),
    "absorbing": dict(kinds=("absorbing",) * 3, absorbing_joint=True),
    "absorbing_m7": dict(kinds=("absorbing",) * 3, absorbing_joint=True, outside_value=-7.0),
    "mixed_prc": dict(kinds=("periodic", "reflective", "clamping")),
    "mixed_ab": dict(kinds=("absorbing", "periodic", "reflective")),
}


def inlet_case(B, axis, positive):
    conc = [9, 17, 5]
    others = [i for i in range(3) if i != axis]
    lats = [np.linspace(B[0, i], B[1, i], conc[i], dtype=F32) for i in others]
    return dict(inlet_axis=axis, inlet_positive=positive, lattices=lats)


@pytest.mark.parametrize("name", list(CASES) + ["inlet_xpos", "inlet_yneg", "inlet_zpos"])
def test_boundaries(golden, name):
    g = golden("boundary")
    B = g["B"]
    if name.startswith("inlet"):
        axis = {"x": 0, "y": 1, "z": 2}[name[6]]
        spec = oracle.BoundarySpec(bounds=B, **inlet_case(B, axis, name.endswith("pos")))
        P = g["Pin"]
    else:
        spec = oracle.BoundarySpec(bounds=B, **CASES[name])
        P = g["P"]
    assert same(oracle.boundary_apply(spec, P), g[name])


@pytest.mark.parametrize("integ", ["rk4", "rk2", "euler"])
def test_track_grid(golden, integ):
    g = golden("track_grid")
    spec = oracle.GridSpec(g["D"], g["st"], g["g"], g["g"], g["g"], "periodic")
    bc = oracle.BoundarySpec(kinds=("periodic",) * 3)
    ref = g[f"{integ}_traj"]
    T = ref.shape[0]
    times = np.linspace(0.0, 0.3 if integ == "rk4" else 0.2, T, dtype=F32)
    out, traj, info = oracle.track(spec, bc, g["x0"], times, 0.01, integ, record=True)
    assert info["wrapped_count"] == 0
    assert same(traj, ref)


def test_track_inlet(golden):
    g = golden("track_inlet")
    spec = oracle.GridSpec(g["D"], g["st"], g["g"], g["g"], g["g"], "clamp")
    lats = [np.linspace(F32(0), F32(1), 16, dtype=F32)] * 2
    bc = oracle.BoundarySpec(inlet_axis=0, inlet_positive=True, lattices=lats)
    times = np.linspace(0.0, 0.6, 61, dtype=F32)
    out, traj, _ = oracle.track(spec, bc, g["x0"], times, 0.01, "rk4", record=True)
    ref = g["traj"]
    assert same(traj, ref)
    # the run must exercise the replacement
    assert np.any(np.diff(ref[:, :, 0], axis=0) < -0.5)


def test_nearest_sampling(golden):
    g = golden("nearest")
    spec = oracle.NearestSpec(g["D"], g["st"], g["nodes"])
    for i, t in enumerate((0.0, 0.7, 2.5, 3.5)):
        out, _ = oracle.sample(spec, g["q"], t, t_is_f32=False)
        # the reference's NumPy path picks nodes with scipy cKDTree (float64
        # distances); away from near-ties the pick is the same node
        assert np.mean(np.all(out == g["outs"][i], axis=1)) > 0.99


def test_quick_scenario(golden):
    """tests/test_quick.py of the reference: 2-D vortex, NN field, reflective, RK4."""
    g = golden("nearest")
    spec = oracle.NearestSpec(g["vort"], g["vt"], g["qn"])
    bc = oracle.BoundarySpec(kinds=("reflective",) * 3, bounds=((-1, -1, -1), (1, 1, 1)))
    times = np.linspace(0.0, 2.0, 101, dtype=F32)
    out, traj, _ = oracle.track(spec, bc, g["seeds"], times, 0.02, "rk4", record=True)
    assert np.allclose(traj, g["quick_traj"], atol=1e-6)


def test_octree_known_answer(golden):
    g = golden("octree")
    assert np.allclose(g["ka_out"], [[0.25, 0.25, 0.25]])


def octree_spec(g):
    return oracle.MeshSpec(g["D"], g["st"], g["P"], g["T4"], g["element_bounds"], g["nodes_min"], g["nodes_max"],
                           g["nodes_elements"], g["nodes_children"], g["nodes_is_leaf"], max_depth=12)


def test_octree_sampling(golden):
    g = golden("octree")
    spec = octree_spec(g)
    for key, t in (("sample_t03", 0.3), ("sample_t10", 1.0)):
        out, fb = oracle.sample(spec, g["q"], float(F32(t)), t_is_f32=True)
        ref = g[key]
        assert np.allclose(out, ref, rtol=1e-5, atol=1e-6), np.abs(out - ref).max()
        assert fb > 0  # the reference's cheap fallback is exercised


def test_octree_tracking(golden):
    g = golden("octree")
    spec = octree_spec(g)
    bc = oracle.BoundarySpec(kinds=("periodic", "reflective", "periodic"))
    times = np.linspace(0.0, 0.1, 11, dtype=F32)
    out, traj, _ = oracle.track(spec, bc, g["x0"], times, 0.01, "rk4", record=True)
    assert np.allclose(traj, g["traj"], rtol=1e-5, atol=1e-6)


# ---------------------------------------------------------------- FEM hash grid
def fem_spec(g):
    return oracle.FemSpec(g["D"], g["st"], g["P"], g["T4"], g["grid_size"], g["grid_min"], g["grid_cell_size"],
                          g["cell_to_elements"], g["element_bounds"])


def test_fem_known_answer(golden):
    g = golden("fem")
    # (0.5,0.5,0.5) lies in neither tet: the nearest node, first of 8 ties (node 0)
    assert np.allclose(g["ka_out"], [[0.0, 0.0, 0.0], [0.1, 0.1, 0.1]])


def test_fem_sampling(golden):
    g = golden("fem")
    spec = fem_spec(g)
    for key, t in (("sample_t03", 0.3), ("sample_t10", 1.0)):
        out, fb = oracle.sample(spec, g["q"], float(F32(t)), t_is_f32=True)
        ref = g[key]
        assert np.allclose(out, ref, rtol=1e-5, atol=1e-6), np.abs(out - ref).max()
        assert fb > 0  # queries outside the mesh take the global nearest node


def test_fem_tracking(golden):
    g = golden("fem")
    spec = fem_spec(g)
    bc = oracle.BoundarySpec(kinds=("periodic", "reflective", "periodic"), bounds=((0, 0, 0), (1, 1, 0.5)))
    times = np.linspace(0.0, 0.08, 9, dtype=F32)
    out, traj, _ = oracle.track(spec, bc, g["x0"], times, 0.01, "rk4", record=True)
    assert np.allclose(traj, g["traj"], rtol=1e-5, atol=1e-6), np.abs(traj - g["traj"]).max()
