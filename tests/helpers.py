"""Shared helpers of the parity tests (seeded inputs, comparisons)."""
from __future__ import annotations

import numpy as np

from gravity_gb300 import abi, ic


def plummer_case(n, seed=0, dead_frac=0.0, nan_count=0, outliers=0):
    b = ic.plummer(n, seed=seed)
    rng = np.random.default_rng(seed + 100)
    if dead_frac:
        dead = rng.choice(n, int(n * dead_frac), replace=False)
        b["pos_mass"][dead, 3] = 0.0
    if nan_count:
        idx = rng.choice(n, nan_count, replace=False)
        b["pos_mass"][idx, 0] = np.nan
    if outliers:
        idx = rng.choice(n, outliers, replace=False)
        b["pos_mass"][idx, :3] *= 1000.0
    return b


def bounds_of(b):
    live = (b["pos_mass"][:, 3] != 0) & np.all(np.isfinite(b["pos_mass"][:, :3]), axis=1)
    p = b["pos_mass"][live, :3]
    return np.concatenate([p.min(0), p.max(0)]).astype(np.float32)


def make_pair(O, BH, bodies, bounds, units=None):
    units = units if units is not None else abi.units(G=1.0)
    g = BH(len(bodies), bounds, units)
    o = O.OracleBarnesHut(len(bodies), bounds, units)
    for x in (g, o):
        x.upload_bodies(bodies)
        x.init()
    return g, o


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b, axis=-1) / np.maximum(np.linalg.norm(b, axis=-1), 1e-30)


def sim_bounds(s):
    return np.array(list(s.bounds_min) + list(s.bounds_max), dtype=np.float32)
