"""The adjoint RK4 kernel against central finite differences of the float64
oracle.  The trilinear field is C0 with derivative jumps on cell faces; a
finite difference that straddles a face differs from the exact derivative.
The oracle reports which differences kept every field evaluation in the
unperturbed run's cells (oracle.fd): those must agree closely, the rest only
in the majority.  On a field whose trilinear interpolant is a global
polynomial (smooth across faces) every difference must agree."""
import numpy as np
import pytest

import jaxtrace_gb300 as jt
import oracle
import oracle.fd as FD
from jaxtrace_gb300 import workloads as W
from jaxtrace_gb300.adjoint import AdjointRK4

pytestmark = pytest.mark.gpu
F32 = np.float32


def _setup(n=16, n_snap=6, npart=256, seed=3):
    g = (np.arange(n) / n).astype(F32)
    st = np.linspace(0, 1, n_snap).astype(F32)
    data = W.abc_snapshots(W.grid_nodes(g, g, g), st)
    rng = np.random.default_rng(seed)
    x0 = rng.random((npart, 3)).astype(F32)
    y = rng.random((npart, 3)).astype(np.float64)
    return g, st, data, x0, y


def _oracle_final(spec, x0, times, dt):
    out, _, _ = oracle.track(spec, oracle.BoundarySpec(kinds=("periodic",) * 3), x0, times, dt,
                             precision=oracle.ORC_F64)
    return out


def _score(ad, fd):
    rel = np.abs(ad - fd) / np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
    return float(np.mean(rel < 1e-3)), float(np.median(rel))


@pytest.mark.parametrize("sort_min", [1 << 30, 0])
def test_adjoint_gradients_match_finite_differences(sort_min):
    """sort_min 0: particles re-sorted by cell at every checkpoint."""
    import torch
    g, st, data, x0, y = _setup()
    T, steps, dt = 31, 30, 0.01
    solver = AdjointRK4(st, g, g, g, "periodic", jt.periodic_boundary(W.UNIT), checkpoint_every=8,
                        sort_bits=3, sort_min_particles=sort_min)
    x0_t = torch.tensor(x0, device="cuda", requires_grad=True)
    U_t = torch.tensor(data.reshape(len(st), 16, 16, 16, 3), device="cuda", requires_grad=True)
    xT = solver(x0_t, U_t, (0.0, 0.3), T, dt=dt)
    # the forward pass is the exact tracking path
    f = jt.StructuredTimeSeriesField(data, st, g, g, g, "periodic")
    ref = jt.create_tracker("rk4", f, jt.periodic_boundary(W.UNIT), record_final_only=True).track_particles(
        x0, (0.0, 0.3), T, dt=dt).positions[-1]
    assert np.array_equal(xT.detach().cpu().numpy(), ref)
    loss = ((xT.double() - torch.tensor(y, device="cuda")) ** 2).sum()
    loss.backward()
    gx = x0_t.grad.cpu().numpy().astype(np.float64)
    gU = U_t.grad.cpu().numpy().reshape(len(st), -1, 3).astype(np.float64)

    spec = oracle.GridSpec(data, st, g, g, g, "periodic")
    times = np.linspace(0.0, 0.3, T, dtype=F32)
    rng = np.random.default_rng(11)
    h = 1e-5
    # dL/dx0: each particle moves alone, so the difference of its own loss term suffices
    picks = [(int(i), int(a)) for i, a in zip(rng.integers(0, len(x0), 48), rng.integers(0, 3, 48))]
    ad, fd = [], []
    for i, a in picks:
        xs = np.repeat(x0[i:i + 1].astype(np.float64), 2, axis=0)
        xs[0, a] += h
        xs[1, a] -= h
        xp, xm = np.float32(xs[0, a]), np.float32(xs[1, a])
        pair = np.repeat(x0[i:i + 1], 2, axis=0)
        pair[0, a], pair[1, a] = xp, xm
        out = _oracle_final(spec, pair, times, dt)
        lp = np.sum((out[0] - y[i]) ** 2)
        lm = np.sum((out[1] - y[i]) ** 2)
        fd.append((lp - lm) / (float(xp) - float(xm)))
        ad.append(gx[i, a])
    frac, med = _score(np.array(ad), np.array(fd))
    assert frac >= 0.85 and med < 1e-4, (frac, med)

    # dL/dU: perturb one snapshot value, rerun every particle
    def full_loss(d):
        s = oracle.GridSpec(d, st, g, g, g, "periodic")
        return np.sum((_oracle_final(s, x0, times, dt) - y) ** 2)

    upicks = [(int(t), int(nd), int(c)) for t, nd, c in zip(rng.integers(0, len(st), 24),
                                                            rng.integers(0, data.shape[1], 24),
                                                            rng.integers(0, 3, 24))]
    # keep entries that some particle actually samples
    ad, fd = [], []
    for t, nd, c in upicks:
        if gU[t, nd, c] == 0.0:
            continue
        dp, dm = data.copy(), data.copy()
        hv = np.float32(1e-3)
        dp[t, nd, c] += hv
        dm[t, nd, c] -= hv
        step = float(dp[t, nd, c]) - float(dm[t, nd, c])
        fd.append((full_loss(dp) - full_loss(dm)) / step)
        ad.append(gU[t, nd, c])
    if ad:
        frac, med = _score(np.array(ad), np.array(fd))
        assert frac >= 0.85 and med < 1e-3, (frac, med)


def test_adjoint_reflective_and_segments():
    """Reflective walls (the cotangent flips sign on a fold) and a last segment
    shorter than the checkpoint interval."""
    import torch
    g, st, data, x0, y = _setup(n=12, npart=128, seed=4)
    g = np.linspace(0, 1, 12).astype(F32)
    data = W.abc_snapshots(W.grid_nodes(g, g, g), st)
    bc = jt.reflective_boundary(W.UNIT)
    solver = AdjointRK4(st, g, g, g, "clamp", bc, checkpoint_every=7)
    x0_t = torch.tensor(x0, device="cuda", requires_grad=True)
    U_t = torch.tensor(data.reshape(len(st), 12, 12, 12, 3), device="cuda", requires_grad=True)
    xT = solver(x0_t, U_t, (0.0, 0.2), 21, dt=0.01)
    loss = ((xT.double() - torch.tensor(y, device="cuda")) ** 2).sum()
    loss.backward()
    gx = x0_t.grad.cpu().numpy().astype(np.float64)
    spec = oracle.GridSpec(data, st, g, g, g, "clamp")
    times = np.linspace(0.0, 0.2, 21, dtype=F32)
    obc = oracle.BoundarySpec(kinds=("reflective",) * 3)
    ad, fd = [], []
    for i in range(0, 128, 4):
        for a in range(3):
            pair = np.repeat(x0[i:i + 1], 2, axis=0)
            xp, xm = np.float32(float(x0[i, a]) + 1e-5), np.float32(float(x0[i, a]) - 1e-5)
            pair[0, a], pair[1, a] = xp, xm
            out, _, _ = oracle.track(spec, obc, pair, times, 0.01, precision=oracle.ORC_F64)
            fd.append((np.sum((out[0] - y[i]) ** 2) - np.sum((out[1] - y[i]) ** 2)) / (float(xp) - float(xm)))
            ad.append(gx[i, a])
    frac, med = _score(np.array(ad), np.array(fd))
    assert frac >= 0.85 and med < 1e-4, (frac, med)


def test_adjoint_position_gradient_alone_and_sorted_agree():
    """dL/dx0 without a snapshot gradient equals the one computed with it, the
    cell-sorted and unsorted runs give the same forward positions, and the
    backward on float32 stage fields gives the same bits as on pair records
    (the stage fields are blended with the same arithmetic)."""
    import torch
    g, st, data, x0, y = _setup(npart=3000, seed=8)
    outs = []
    for sort_min, need_u, stage in ((1 << 30, True, False), (0, True, True), (0, False, True)):
        solver = AdjointRK4(st, g, g, g, "periodic", jt.periodic_boundary(W.UNIT), checkpoint_every=9,
                            sort_bits=4, sort_min_particles=sort_min, stage_fields=stage)
        x0_t = torch.tensor(x0, device="cuda", requires_grad=True)
        U_t = torch.tensor(data.reshape(len(st), 16, 16, 16, 3), device="cuda", requires_grad=need_u)
        xT = solver(x0_t, U_t, (0.0, 0.25), 26, dt=0.01)
        ((xT - torch.tensor(y, device="cuda", dtype=torch.float32)) ** 2).sum().backward()
        outs.append((xT.detach().cpu().numpy(), x0_t.grad.cpu().numpy(),
                     U_t.grad.cpu().numpy() if need_u else None))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[1][0], outs[2][0])
    # same per-particle arithmetic: dL/dx0 identical bit for bit
    assert np.array_equal(outs[0][1], outs[1][1]) and np.array_equal(outs[1][1], outs[2][1])
    # dL/dU: float atomics in a different order
    assert np.allclose(outs[0][2], outs[1][2], rtol=1e-4, atol=1e-6 * np.abs(outs[0][2]).max())


def test_adjoint_matches_float64_differences_below_float32_resolution():
    """With float64 start points and h = 1e-7 almost no difference straddles a
    cell face, so dL/dx0 must agree closely: 95 % within 1e-4 relative."""
    import torch
    g, st, data, x0, y = _setup(npart=128, seed=12)
    solver = AdjointRK4(st, g, g, g, "periodic", jt.periodic_boundary(W.UNIT), checkpoint_every=10)
    x0_t = torch.tensor(x0, device="cuda", requires_grad=True)
    U_t = torch.tensor(data.reshape(len(st), 16, 16, 16, 3), device="cuda")
    xT = solver(x0_t, U_t, (0.0, 0.2), 21, dt=0.01)
    ((xT.double() - torch.tensor(y, device="cuda")) ** 2).sum().backward()
    gx = x0_t.grad.cpu().numpy().astype(np.float64)
    spec = oracle.GridSpec(data, st, g, g, g, "periodic")
    times = np.linspace(0.0, 0.2, 21, dtype=F32)
    h = 1e-7
    ad, fd = [], []
    for i in range(0, 128, 2):
        for a in range(3):
            pair = np.repeat(x0[i:i + 1].astype(np.float64), 2, axis=0)
            pair[0, a] += h
            pair[1, a] -= h
            out = _oracle_final(spec, pair, times, 0.01)
            fd.append((np.sum((out[0] - y[i]) ** 2) - np.sum((out[1] - y[i]) ** 2)) / (2 * h))
            ad.append(gx[i, a])
    ad, fd = np.array(ad), np.array(fd)
    rel = np.abs(ad - fd) / np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
    assert np.mean(rel < 1e-4) >= 0.95, (np.mean(rel < 1e-4), np.median(rel))


def _polynomial_field(n=12, n_snap=4):
    """Snapshots of a velocity field that is trilinear in space and linear in
    time, on a grid over [-1, 2]^3: trilinear interpolation reproduces it
    exactly, so the field (and the flow map) is smooth across cell faces."""
    g = np.linspace(-1.0, 2.0, n).astype(F32)
    P = W.grid_nodes(g, g, g).astype(np.float64)
    x, yy, z = P[:, 0], P[:, 1], P[:, 2]
    base = np.stack([0.2 + 0.3 * yy - 0.2 * z + 0.4 * yy * z,
                     -0.1 + 0.25 * x + 0.3 * z - 0.3 * x * z,
                     0.15 - 0.2 * x + 0.35 * yy + 0.2 * x * yy], axis=1)
    st = np.linspace(0.0, 1.0, n_snap).astype(F32)
    data = np.stack([base * (1.0 + 0.5 * float(t)) for t in st]).astype(F32)
    return g, st, data


def test_adjoint_matches_differences_on_a_field_smooth_across_faces():
    """Global trilinear-in-space, linear-in-time field, clamp sampler, no
    boundary, particles that stay inside: 99 % of dL/dx0 (h = 1e-4, float64
    start points) and of dL/dU (h = 1e-3) within 1e-4 relative."""
    import torch
    g, st, data = _polynomial_field()
    rng = np.random.default_rng(21)
    x0 = rng.uniform(0.25, 0.75, (256, 3)).astype(F32)
    y = rng.random((256, 3))
    T, dt = 41, 0.01
    solver = AdjointRK4(st, g, g, g, "clamp", None, checkpoint_every=16)
    x0_t = torch.tensor(x0, device="cuda", requires_grad=True)
    U_t = torch.tensor(data.reshape(len(st), 12, 12, 12, 3), device="cuda", requires_grad=True)
    xT = solver(x0_t, U_t, (0.0, 0.4), T, dt=dt)
    ((xT.double() - torch.tensor(y, device="cuda")) ** 2).sum().backward()
    gx = x0_t.grad.cpu().numpy().astype(np.float64)
    gU = U_t.grad.cpu().numpy().reshape(len(st), -1, 3).astype(np.float64)
    spec = oracle.GridSpec(data, st, g, g, g, "clamp")
    obc = oracle.BoundarySpec(kinds=("none",) * 3)
    times = np.linspace(0.0, 0.4, T, dtype=F32)
    picks = [(i, a) for i in range(0, 256, 2) for a in range(3)]
    fd, same = FD.dx0_differences(spec, obc, x0, y, picks, times, dt, 1e-4, f64_start=True)
    ad = np.array([gx[i, a] for i, a in picks])
    a = FD.agreement(ad, fd, same, tol=1e-4)
    assert a["frac_within"] >= 0.99, a
    nz = np.argwhere(gU != 0.0)
    sel = nz[rng.choice(len(nz), size=min(64, len(nz)), replace=False)]
    fdu, sameu = FD.du_differences(spec, obc, x0[:64], y[:64], [tuple(v) for v in sel], times, dt, h=1e-3)
    # the adjoint of the 64-particle loss
    x0_s = torch.tensor(x0[:64], device="cuda")
    U_s = U_t.detach().clone().requires_grad_(True)
    xs = solver(x0_s, U_s, (0.0, 0.4), T, dt=dt)
    ((xs.double() - torch.tensor(y[:64], device="cuda")) ** 2).sum().backward()
    gUs = U_s.grad.cpu().numpy().reshape(len(st), -1, 3).astype(np.float64)
    adu = np.array([gUs[t, nd, c] for t, nd, c in sel])
    keep = fdu != 0.0
    a = FD.agreement(adu[keep], fdu[keep], sameu[keep], tol=1e-4)
    assert a["frac_within"] >= 0.99, a


def test_adjoint_agrees_where_differences_keep_their_cells():
    """ABC field (faces matter): over the differences whose runs kept every
    field evaluation in the unperturbed cells, 99 % of dL/dx0 agree within
    1e-3 at h = 1e-5; the face-crossing ones are what the overall share
    loses."""
    import torch
    g, st, data, x0, y = _setup(npart=512, seed=5)
    T, dt = 41, 0.01
    solver = AdjointRK4(st, g, g, g, "periodic", jt.periodic_boundary(W.UNIT), checkpoint_every=10)
    x0_t = torch.tensor(x0, device="cuda", requires_grad=True)
    U_t = torch.tensor(data.reshape(len(st), 16, 16, 16, 3), device="cuda")
    xT = solver(x0_t, U_t, (0.0, 0.4), T, dt=dt)
    ((xT.double() - torch.tensor(y, device="cuda")) ** 2).sum().backward()
    gx = x0_t.grad.cpu().numpy().astype(np.float64)
    spec = oracle.GridSpec(data, st, g, g, g, "periodic")
    obc = oracle.BoundarySpec(kinds=("periodic",) * 3)
    times = np.linspace(0.0, 0.4, T, dtype=F32)
    picks = [(i, a) for i in range(512) for a in range(3)]
    fd, same = FD.dx0_differences(spec, obc, x0, y, picks, times, dt, 1e-5)
    ad = np.array([gx[i, a] for i, a in picks])
    a = FD.agreement(ad, fd, same)
    assert a["same_cells"]["samples"] > 0.5 * len(picks), a
    assert a["same_cells"]["frac_within"] >= 0.99, a
