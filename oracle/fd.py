"""Central finite differences of the float64 oracle, the check of the adjoint
RK4 kernel -- TEST INFRASTRUCTURE ONLY (imported by tests/ and by bench.py's
adjoint check, never by the package).

A trilinear field is continuous with derivative jumps on cell faces, so the
flow map is smooth only while a trajectory stays in the same sequence of
cells.  Each difference therefore also reports whether its two perturbed
runs evaluated the field in exactly the cells of the unperturbed run (the
oracle's cell signature): where they did, the difference approximates the
derivative the adjoint computes to O(h^2); where they did not, it straddles a
face and measures a chord across the derivative jump instead.
"""
from __future__ import annotations

import numpy as np

from . import ORC_F64, track


def _sq_loss(out, y):
    return np.sum((out - y) ** 2, axis=1)


def dx0_differences(spec, boundary, x0, y, picks, times, dt, h, f64_start=False, n_threads=0):
    """d L_i / d x0[i, a] for picks [(i, a)], L_i = |x_T(x0_i) - y_i|^2 (each
    particle moves alone, so its own loss term is the whole difference).

    float32 start points (the adjoint's own) perturbed to the nearest float32
    values, or with ``f64_start`` float64 start points perturbed by h exactly.
    Returns (differences (k,), same_cells (k,) bool)."""
    picks = list(picks)
    k = len(picks)
    idx = np.array([i for i, _ in picks], dtype=np.int64)
    ax = np.array([a for _, a in picks], dtype=np.int64)
    r = np.arange(k)
    if f64_start:
        base = np.asarray(x0, np.float64)[idx]
        plus, minus = base.copy(), base.copy()
        plus[r, ax] += h
        minus[r, ax] -= h
    else:
        base = np.asarray(x0, np.float32)[idx]
        plus, minus = base.copy(), base.copy()
        plus[r, ax] = (base[r, ax].astype(np.float64) + h).astype(np.float32)
        minus[r, ax] = (base[r, ax].astype(np.float64) - h).astype(np.float32)
    X = np.concatenate([base, plus, minus]).astype(np.float64)
    out, _, info = track(spec, boundary, X, times, dt, precision=ORC_F64, n_threads=n_threads, cell_sig=True)
    yk = np.asarray(y, np.float64)[idx]
    step = plus[r, ax].astype(np.float64) - minus[r, ax].astype(np.float64)
    fd = (_sq_loss(out[k:2 * k], yk) - _sq_loss(out[2 * k:], yk)) / step
    sig = info["cell_sig"]
    same = (sig[k:2 * k] == sig[:k]) & (sig[2 * k:] == sig[:k])
    return fd, same


def du_differences(spec, boundary, x0, y, picks, times, dt, h=1e-3, n_threads=0):
    """d L / d U[t, node, c] for picks [(t, node, c)], L = sum_i |x_T,i - y_i|^2
    over the particles x0, with the snapshot value moved by +-h in float32
    (in place in ``spec``'s own data array, restored after each pick).
    Returns (differences (k,), same_cells (k,) bool: every particle of both
    runs visited the cells of the unperturbed run)."""
    data = spec.keep[0]
    _, _, info = track(spec, boundary, x0, times, dt, precision=ORC_F64, n_threads=n_threads, cell_sig=True)
    base_sig = info["cell_sig"]
    yy = np.asarray(y, np.float64)
    hv = np.float32(h)
    fd, same = [], []
    for t, nd, c in picks:
        v0 = data[t, nd, c]
        data[t, nd, c] = v0 + hv
        vp = float(data[t, nd, c])
        op, _, ip = track(spec, boundary, x0, times, dt, precision=ORC_F64, n_threads=n_threads, cell_sig=True)
        data[t, nd, c] = v0 - hv
        vm = float(data[t, nd, c])
        om, _, im = track(spec, boundary, x0, times, dt, precision=ORC_F64, n_threads=n_threads, cell_sig=True)
        data[t, nd, c] = v0
        fd.append((np.sum(_sq_loss(op, yy)) - np.sum(_sq_loss(om, yy))) / (vp - vm))
        same.append(bool(np.array_equal(ip["cell_sig"], base_sig) and np.array_equal(im["cell_sig"], base_sig)))
    return np.array(fd), np.array(same, dtype=bool)


def agreement(ad, fd, same=None, tol=1e-3):
    """Relative difference |ad - fd| / max(|fd|, 1e-3 max|fd|): the share
    within ``tol`` and the median, over all samples and (given ``same``)
    over those whose runs kept their cells and those that crossed a face."""
    ad, fd = np.asarray(ad, np.float64), np.asarray(fd, np.float64)
    rel = np.abs(ad - fd) / np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())

    def summ(m):
        if not np.any(m):
            return {"samples": 0, "frac_within": None, "median_rel": None}
        return {"samples": int(m.sum()), "frac_within": float(np.mean(rel[m] < tol)),
                "median_rel": float(np.median(rel[m]))}

    out = summ(np.ones(len(rel), bool))
    out["tol"] = tol
    if same is not None:
        same = np.asarray(same, bool)
        out["same_cells"] = summ(same)
        out["crossing_a_face"] = summ(~same)
    return out
