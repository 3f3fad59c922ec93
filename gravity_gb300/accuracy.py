"""Acceleration error of a walk against the direct-sum reference, and matching of
acceptance settings at equal p99 error.

The judge (gbh_direct_sum) is an FP64 direct sum: every live body's pull on a
seeded sample of bodies, FP64 terms and FP64 sums.  Errors are
|a_walk - a_direct| / |a_direct| per sampled body.
"""
from __future__ import annotations

import numpy as np

from . import abi


def sample_bodies(n_live_ids: np.ndarray, count: int = 4096, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    k = min(count, len(n_live_ids))
    return np.sort(rng.choice(n_live_ids, k, replace=False)).astype(np.uint32)


def live_ids(sim) -> np.ndarray:
    b = sim.read_bodies()
    return np.nonzero(b["pos_mass"][:, 3] != 0)[0].astype(np.uint32)


class DirectSumSample:
    """FP64 direct-sum accelerations of a fixed sample of the current state."""

    judge = "fp64"

    def __init__(self, sim, params: abi.StepParams, count: int = 4096, seed: int = 0):
        self.sample = sample_bodies(live_ids(sim), count, seed)
        self.ref = sim.direct_sum(params, self.sample)

    def errors(self, accel: np.ndarray) -> np.ndarray:
        a = np.asarray(accel, np.float64)[self.sample]
        return np.linalg.norm(a - self.ref, axis=1) / np.maximum(np.linalg.norm(self.ref, axis=1), 1e-300)


def summarize(err: np.ndarray) -> dict:
    return {
        "median": float(np.median(err)),
        "p90": float(np.percentile(err, 90)),
        "p99": float(np.percentile(err, 99)),
        "max": float(np.max(err)),
    }


def evaluate(sim, ref_sample: DirectSumSample, params: abi.StepParams) -> dict:
    """Error summary and interactions of one walk of the current state."""
    acc = sim.evaluate_walk(params)
    s = sim.read_stats()
    out = summarize(ref_sample.errors(acc))
    out["interactions"] = int(s.interactions)
    out["mac_evaluations"] = int(s.mac_evaluations)
    return out


def match_p99(sim, ref_sample: DirectSumSample, make_params, grid, target_p99: float, refine: int = 0):
    """The setting of `grid` (ordered from accurate to aggressive) with the
    fewest interactions whose p99 error stays at or below `target_p99`.
    With `refine` > 0, when the grid's next (more aggressive) setting after
    that one misses the target, `refine` bisection steps between the two look
    for a setting closer to the target.  Returns (value, result dict, all
    results)."""
    results = []
    best = None

    def run(v):
        nonlocal best
        r = evaluate(sim, ref_sample, make_params(v))
        r["setting"] = float(v)
        results.append(r)
        if r["p99"] <= target_p99 and (best is None or r["interactions"] < best[1]["interactions"]):
            best = (float(v), r)
        return r

    for v in grid:
        run(v)
    if refine and best is not None:
        settings = [float(v) for v in grid]
        i = settings.index(best[0])
        if i + 1 < len(settings) and results[i + 1]["p99"] > target_p99:
            lo, hi = settings[i], settings[i + 1]
            for _ in range(refine):
                mid = 0.5 * (lo + hi)
                if run(mid)["p99"] <= target_p99:
                    lo = mid
                else:
                    hi = mid
    return best, results
