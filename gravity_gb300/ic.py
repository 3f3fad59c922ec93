"""Seeded initial conditions for the benchmark workloads.

The reference's own generators (PlanetGenerator.java:310-484) draw from an
unseeded Math.random() and only build disks and boxes, so the workloads here
are generated by this module from a numpy PCG64 stream with a fixed seed.  All
outputs are arrays of the reference Body layout (abi.BODY_DTYPE, 32 bytes).

Workloads (sizes are the defaults; every generator takes n):
  plummer            Plummer sphere, scale radius a, equal masses total_mass/n,
                     isotropic velocities from the Plummer distribution
                     function (Aarseth, Henon & Wielen 1974 rejection sampling).
  uniform_merge      n bodies uniform in [-1,1]^3, masses log-uniform in
                     [1e-6, 1e-3], zero velocity, density chosen so that the
                     reference radius formula gives r = 0.002 (m/1e-3)^(1/3).
  plummer_uniform    70% Plummer (a=1) + 30% uniform in [-3,3]^3 at rest,
                     equal masses 1/n.
  galaxy_pair        two galaxies, each 80% exponential disk (R_d=1, z_d=0.1)
                     and 20% Hernquist bulge (a=0.2), separated by 10 on a
                     parabolic orbit, equal-mass particles.
  cluster_mixture    Gaussian clusters (sigma log-uniform in [0.01, 0.1],
                     centres uniform in [-10,10]^3), power-law masses
                     dN/dm ~ m^-2 on [1e-9, 1e-6], at rest.
"""
from __future__ import annotations

import numpy as np

from . import abi

# radius(Body) = 0.6203504909 (m/rho)^(1/3) with unit mass/density/length 1
# (common.glsl:228-230, 346-352); r = 0.002 (m/1e-3)^(1/3)  <=>  rho below.
MERGE_DENSITY = (0.6203504909 / 0.002) ** 3 * 1e-3


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _unit_vectors(rng, n):
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


def pack(pos, vel, mass, density) -> np.ndarray:
    n = len(mass)
    out = np.zeros(n, dtype=abi.BODY_DTYPE)
    out["pos_mass"][:, :3] = pos
    out["pos_mass"][:, 3] = mass
    out["vel_density"][:, :3] = vel
    out["vel_density"][:, 3] = density
    return out


def plummer_arrays(n, rng, a=1.0, total_mass=1.0, G=1.0, max_mass_fraction=0.999):
    x1 = rng.uniform(0.0, max_mass_fraction, n)
    x1 = np.maximum(x1, 1e-12)
    r = a / np.sqrt(x1 ** (-2.0 / 3.0) - 1.0)
    pos = _unit_vectors(rng, n) * r[:, None]
    # speed fraction q from g(q) = q^2 (1-q^2)^(7/2), rejection sampling
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        x4 = rng.uniform(0.0, 1.0, todo.size)
        x5 = rng.uniform(0.0, 0.1, todo.size)
        ok = x5 < x4 * x4 * (1.0 - x4 * x4) ** 3.5
        q[todo[ok]] = x4[ok]
        todo = todo[~ok]
    vesc = np.sqrt(2.0 * G * total_mass / a) * (1.0 + (r / a) ** 2) ** (-0.25)
    vel = _unit_vectors(rng, n) * (q * vesc)[:, None]
    mass = np.full(n, total_mass / n)
    return pos, vel, mass


def plummer(n=65536, seed=0, a=1.0, G=1.0) -> np.ndarray:
    """Plummer sphere, the small plain-method workload (65,536 bodies, seed 0)."""
    rng = _rng(seed)
    pos, vel, mass = plummer_arrays(n, rng, a=a, G=G)
    return pack(pos, vel, mass, np.ones(n))


def uniform_merge(n=1048576, seed=1) -> np.ndarray:
    """Uniform cube with merges and out-of-bounds kills (1,048,576 bodies)."""
    rng = _rng(seed)
    pos = rng.uniform(-1.0, 1.0, (n, 3))
    mass = 10.0 ** rng.uniform(-6.0, -3.0, n)
    return pack(pos, np.zeros((n, 3)), mass, np.full(n, MERGE_DENSITY))


def plummer_uniform(n=16777216, seed=3, plummer_fraction=0.7, cube=3.0) -> np.ndarray:
    """70/30 Plummer + uniform mixture (16,777,216 bodies), equal masses 1/n."""
    rng = _rng(seed)
    n_p = int(round(n * plummer_fraction))
    n_u = n - n_p
    pos_p, vel_p, _ = plummer_arrays(n_p, rng, a=1.0, total_mass=1.0)
    pos_u = rng.uniform(-cube, cube, (n_u, 3))
    pos = np.concatenate([pos_p, pos_u])
    vel = np.concatenate([vel_p, np.zeros((n_u, 3))])
    perm = rng.permutation(n)
    return pack(pos[perm], vel[perm], np.full(n, 1.0 / n), np.ones(n))


def _galaxy(n, rng, G=1.0, mass=1.0):
    n_disk = int(round(0.8 * n))
    n_bulge = n - n_disk
    m_bulge, m_disk = 0.2 * mass, 0.8 * mass
    # exponential disk: R ~ Gamma(2, R_d), z ~ Laplace(z_d)
    R = rng.gamma(2.0, 1.0, n_disk)
    phi = rng.uniform(0.0, 2.0 * np.pi, n_disk)
    z = rng.laplace(0.0, 0.1, n_disk)
    pos_d = np.stack([R * np.cos(phi), R * np.sin(phi), z], axis=1)
    # Hernquist bulge, a = 0.2: M(<r)/M = r^2/(r+a)^2
    x = rng.uniform(0.0, 0.999, n_bulge)
    s = np.sqrt(x)
    rb = 0.2 * s / (1.0 - s)
    pos_b = _unit_vectors(rng, n_bulge) * rb[:, None]
    # circular speed of the disk from the enclosed mass of both components
    m_enc_disk = m_disk * (1.0 - np.exp(-R) * (1.0 + R))
    m_enc_bulge = m_bulge * R * R / (R + 0.2) ** 2
    vc = np.sqrt(G * (m_enc_disk + m_enc_bulge) / np.maximum(R, 1e-3))
    vel_d = np.stack([-vc * np.sin(phi), vc * np.cos(phi), np.zeros(n_disk)], axis=1)
    vel_d += rng.normal(0.0, 0.05, (n_disk, 3)) * vc[:, None]
    # bulge: isotropic Gaussian velocities with sigma^2 = G M(<r) / (3 r)
    m_enc = m_bulge * rb * rb / (rb + 0.2) ** 2 + m_disk * (1.0 - np.exp(-rb) * (1.0 + rb))
    sig = np.sqrt(G * m_enc / (3.0 * np.maximum(rb, 1e-3)))
    vel_b = rng.normal(0.0, 1.0, (n_bulge, 3)) * sig[:, None]
    return np.concatenate([pos_d, pos_b]), np.concatenate([vel_d, vel_b])


def galaxy_pair(n_per_galaxy=4194304, seed=2, separation=10.0, pericentre=1.5, G=1.0) -> np.ndarray:
    """Two-galaxy merger on a parabolic orbit (2 x 4,194,304 bodies)."""
    rng = _rng(seed)
    p1, v1 = _galaxy(n_per_galaxy, rng, G=G)
    p2, v2 = _galaxy(n_per_galaxy, rng, G=G)
    # tilt the second disk by 60 degrees about x
    c, s = np.cos(np.pi / 3), np.sin(np.pi / 3)
    rot = np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    p2 = p2 @ rot.T
    v2 = v2 @ rot.T
    m_tot = 2.0
    v_rel = np.sqrt(2.0 * G * m_tot / separation)
    sin_phi = np.sqrt(pericentre / separation)
    cos_phi = np.sqrt(1.0 - sin_phi * sin_phi)
    rel_v = np.array([-v_rel * cos_phi, v_rel * sin_phi, 0.0])
    p1 = p1 + np.array([-separation / 2, 0, 0])
    p2 = p2 + np.array([separation / 2, 0, 0])
    v1 = v1 - rel_v / 2
    v2 = v2 + rel_v / 2
    n = 2 * n_per_galaxy
    pos = np.concatenate([p1, p2])
    vel = np.concatenate([v1, v2])
    return pack(pos, vel, np.full(n, m_tot / n), np.ones(n))


def cluster_mixture(n=33554432, seed=4, clusters=256) -> np.ndarray:
    """Gaussian mixture of clusters with power-law masses (33,554,432 bodies)."""
    rng = _rng(seed)
    centres = rng.uniform(-10.0, 10.0, (clusters, 3))
    sig = 10.0 ** rng.uniform(-2.0, -1.0, clusters)
    which = rng.integers(0, clusters, n)
    pos = centres[which] + rng.normal(0.0, 1.0, (n, 3)) * sig[which][:, None]
    lo, hi = 1e-9, 1e-6
    u = rng.uniform(0.0, 1.0, n)
    mass = 1.0 / (1.0 / lo - u * (1.0 / lo - 1.0 / hi))
    return pack(pos, np.zeros((n, 3)), mass, np.full(n, MERGE_DENSITY))


def exact_bounds(bodies: np.ndarray) -> np.ndarray:
    """AABB of the live bodies as [minx, miny, minz, maxx, maxy, maxz] (FP32)."""
    live = bodies["pos_mass"][:, 3] != 0
    p = bodies["pos_mass"][live, :3]
    return np.concatenate([p.min(axis=0), p.max(axis=0)]).astype(np.float32)
