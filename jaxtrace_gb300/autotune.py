"""Autotuner of the tracking pass.

The tracking kernel has three launch-time knobs whose best values depend on
the field, the particle count and their spread: the block size (64, 128 or
256 threads), how often particles are re-sorted by cell (``sort_every``) and
the cell size of that sort (``sort_bits``).  ``Autotuner`` times candidate
settings on a short sample of the real run (every k-th particle of every
ensemble, the first steps of the time grid), keeps the fastest, and caches it
under a key of device, field kind, storage, integrator and problem size, in
memory and optionally in the JSON file named by ``JAXTRACE_GB300_TUNE_CACHE``.

The search is coordinate descent: block size with the default sort, then the
sort interval, then the sort cell size, each stage keeping the previous
stages' winners.  A sample is timed with CUDA events on the current stream
after one untimed warm-up pass.
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass
from typing import Dict, List, Optional, Tuple

BLOCK_SIZES = (128, 256, 64)
SORT_EVERY = (0, 20, 50, 100)
SORT_BITS = (7, 6, 5)


@dataclass
class TuneResult:
    block_size: int
    sort_every: int
    sort_bits: int
    ms: float
    trials: List[Tuple[int, int, int, float]]


def _bucket(n: int) -> int:
    """Particle counts within a factor 2 share a tuning result."""
    return int(max(n, 1)).bit_length()


class Autotuner:
    _shared: Optional["Autotuner"] = None

    def __init__(self, cache_path: Optional[str] = None, sample_particles: int = 1 << 21,
                 sample_steps: int = 100):
        self.cache_path = cache_path if cache_path is not None else os.environ.get("JAXTRACE_GB300_TUNE_CACHE")
        self.sample_particles = int(sample_particles)
        self.sample_steps = int(sample_steps)
        self.cache: Dict[str, dict] = {}
        if self.cache_path and os.path.exists(self.cache_path):
            with open(self.cache_path) as fh:
                self.cache = json.load(fh)

    @classmethod
    def shared(cls) -> "Autotuner":
        if cls._shared is None:
            cls._shared = cls()
        return cls._shared

    # ------------------------------------------------------------------
    def key(self, tracker, n: int, n_steps: int) -> str:
        import torch
        f = tracker._field
        return "|".join([torch.cuda.get_device_name(), type(f).__name__, f.storage, str(tracker._code),
                         "exact" if tracker._arith() == 0 else "compensated", f"n{_bucket(n)}", f"s{_bucket(n_steps)}"])

    def _save(self):
        if self.cache_path:
            tmp = self.cache_path + ".tmp"
            with open(tmp, "w") as fh:
                json.dump(self.cache, fh, indent=1, sort_keys=True)
            os.replace(tmp, self.cache_path)

    def _apply(self, tracker, r: dict):
        o = tracker.options
        o.block_size, o.sort_every, o.sort_bits = int(r["block_size"]), int(r["sort_every"]), int(r["sort_bits"])

    def search(self, tracker, time_sample) -> TuneResult:
        """Coordinate descent over (block_size, sort_every, sort_bits);
        ``time_sample()`` runs the sample once with the tracker's current
        options and returns milliseconds."""
        o = tracker.options
        saved = (o.block_size, o.sort_every, o.sort_bits)
        trials: List[Tuple[int, int, int, float]] = []
        best = [256, 100, 7]

        def trial(bs, se, sb):
            o.block_size, o.sort_every, o.sort_bits = bs, se, sb
            ms = time_sample()
            trials.append((bs, se, sb, ms))
            return ms

        try:
            scores = {bs: trial(bs, best[1], best[2]) for bs in BLOCK_SIZES}
            best[0] = min(scores, key=scores.get)
            scores = {se: trial(best[0], se, best[2]) for se in SORT_EVERY}
            best[1] = min(scores, key=scores.get)
            if best[1] > 0:
                scores = {sb: trial(best[0], best[1], sb) for sb in SORT_BITS}
                best[2] = min(scores, key=scores.get)
        finally:
            o.block_size, o.sort_every, o.sort_bits = saved
        ms = min(t[3] for t in trials if (t[0], t[1], t[2]) == tuple(best))
        return TuneResult(best[0], best[1], best[2], ms, trials)

    # ------------------------------------------------------------------
    def tune_batch(self, batch) -> TuneResult:
        """Tune the options of ``batch.tracker`` for an ``EnsembleBatch``."""
        from .tracker import EnsembleBatch
        tr = batch.tracker
        key = self.key(tr, batch.n, batch.n_steps)
        if key in self.cache:
            self._apply(tr, self.cache[key])
            r = self.cache[key]
            return TuneResult(r["block_size"], r["sort_every"], r["sort_bits"], r["ms"], [])
        stride = max(1, -(-batch.n // self.sample_particles))
        host = batch.x0.cpu().numpy()
        subs = [host[a:b:stride] for a, b in zip(batch.offsets[:-1], batch.offsets[1:])]
        steps = min(batch.n_steps, self.sample_steps)
        rel = [float(t[0]) for t in batch.times]
        sample = EnsembleBatch(tr, subs, rel, steps + 1, dt=batch.dt)
        res = self.search(tr, lambda: _time(sample.run))
        self.cache[key] = {"block_size": res.block_size, "sort_every": res.sort_every,
                           "sort_bits": res.sort_bits, "ms": res.ms, "sample_particles": sample.n,
                           "sample_steps": steps}
        self._save()
        self._apply(tr, self.cache[key])
        return res


def _time(fn, warmup: int = 1) -> float:
    import torch
    for _ in range(warmup):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return float(e0.elapsed_time(e1))


__all__ = ["Autotuner", "TuneResult", "BLOCK_SIZES", "SORT_EVERY", "SORT_BITS"]
