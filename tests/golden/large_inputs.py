"""Inputs of the large golden fixtures (65,536 bodies), regenerated anywhere.

The large fixtures do not store their input bodies: they store the generator's
name and arguments and a SHA-256 of the bodies it produced, and the replay
regenerates them and checks the digest first.  The generator uses only integer
hashing (SplitMix64 on uint64 arrays) and IEEE single-precision +, - and *,
which round the same way on every machine and numpy version.

Outputs of the reference are stored as digests of the exact words (NaN
payloads made canonical first), plus every 16th body after the step for the
comparisons that carry a tolerance.
"""
from __future__ import annotations

import hashlib

import numpy as np

from gravity_gb300 import abi

GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def _splitmix(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + GOLDEN
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniforms(seed: int, stream: int, n: int) -> np.ndarray:
    """n float32 values in [0, 1), exact multiples of 2^-24."""
    with np.errstate(over="ignore"):
        ctr = np.arange(n, dtype=np.uint64) + np.uint64(stream) * np.uint64(0x100000000) + \
            np.uint64(seed) * np.uint64(0x1000000000000)
    return (_splitmix(ctr) >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)


def clusters(n: int, seed: int, k: int = 64, defects: bool = True) -> np.ndarray:
    """k clusters with centres in [-1,1]^3 and radii in [0.01, 0.2); a body
    lies at its centre plus u^3 times a uniform vector in the cluster's cube,
    so the density rises steeply toward each centre (deep trees).  With
    defects: 5% empty bodies, 2 NaN positions and 3 outliers far out."""
    two, one = np.float32(2.0), np.float32(1.0)
    cid = (uniforms(seed, 0, n) * np.float32(k)).astype(np.int64)
    cx, cy, cz = (uniforms(seed, 1 + a, k) * two - one for a in range(3))
    rad = uniforms(seed, 4, k) * np.float32(0.19) + np.float32(0.01)
    u = uniforms(seed, 5, n)
    s = u * u * u * rad[cid]
    b = np.zeros(n, dtype=abi.BODY_DTYPE)
    pm, vd = b["pos_mass"], b["vel_density"]
    for a, c in enumerate((cx, cy, cz)):
        pm[:, a] = c[cid] + (uniforms(seed, 6 + a, n) * two - one) * s
        vd[:, a] = (uniforms(seed, 9 + a, n) * two - one) * np.float32(0.1)
    pm[:, 3] = (uniforms(seed, 12, n) * np.float32(0.9) + np.float32(0.1)) * np.float32(1.0 / n)
    vd[:, 3] = np.float32(1.0)
    if defects:
        d = uniforms(seed, 13, n)
        pm[d < np.float32(0.05), 3] = 0.0
        pm[[17, n // 2 + 5], 0] = np.nan
        pm[[101, 2021, n - 7], :3] *= np.float32(50.0)
    return b


def merge_box(n: int, seed: int) -> np.ndarray:
    """Bodies uniform in [-0.2,0.2]^3 at rest with masses in [1e-6, 1e-3) and
    radius 0.002 (m / 1e-3)^(1/3) through the constant density of the merge
    workload; 8 bodies sit outside the box [-2,2]^3 and are killed."""
    two, one = np.float32(2.0), np.float32(1.0)
    b = np.zeros(n, dtype=abi.BODY_DTYPE)
    pm, vd = b["pos_mass"], b["vel_density"]
    for a in range(3):
        pm[:, a] = (uniforms(seed, a, n) * two - one) * np.float32(0.2)
    pm[:, 3] = uniforms(seed, 3, n) * np.float32(1e-3 - 1e-6) + np.float32(1e-6)
    vd[:, 3] = np.float32((0.6203504909 / 0.002) ** 3 * 1e-3)
    pm[:8, 0] = np.float32(3.0)
    return b


GENERATORS = {"clusters": clusters, "merge_box": merge_box}


def make(kind: str, n: int, seed: int) -> np.ndarray:
    return GENERATORS[kind](n, seed)


def digest(a) -> str:
    """SHA-256 of the words of an array, every float NaN made the canonical
    quiet NaN (CUDA and x86 write different NaN payloads)."""
    a = np.ascontiguousarray(a)
    if a.dtype.fields is None and a.dtype.kind == "f":
        f = a.astype(np.float32, copy=True)
        f[np.isnan(f)] = np.float32(np.nan)
        w = f.view(np.uint32).copy()
        w[np.isnan(f)] = 0x7FC00000
        a = w
    return hashlib.sha256(a.tobytes()).hexdigest()


def node_digests(nodes: np.ndarray) -> dict:
    """Digests of a node array's exact fields (not the render-only colour)."""
    out = {}
    for f in ("child_a", "child_b", "parent_id", "bodies_contained", "node_depth", "ready_children"):
        out[f] = digest(nodes[f])
    for f in ("com_mass", "aabb"):
        out[f] = digest(nodes[f])
    return out


def task_digest(tasks: np.ndarray) -> str:
    """Digest of a merge-task set (order-free: pairs sorted)."""
    t = np.asarray(tasks, np.uint32).reshape(-1, 2)
    key = (t[:, 0].astype(np.uint64) << np.uint64(32)) | t[:, 1].astype(np.uint64)
    return digest(np.sort(key))
