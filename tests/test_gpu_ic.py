"""Seeded initial conditions generated on the device (gbh_generate_bodies).

The box kind is pinned bit for bit against a numpy restatement of the
counter-based generator (splitmix64 of seed * K0 + (i + 1) * K1 + (d + 1) * K2,
top 24 bits, FP32 range map); the other kinds against their defining
properties: Plummer half-mass radius and virial ratio, an in-plane disk with
tangential orbital velocities and its centre body last, clusters around their
centres with masses in range.  Chunked generation must equal one-shot."""
import numpy as np
import pytest

from gravity_gb300 import BarnesHut, abi

pytestmark = pytest.mark.gpu

K0, K1, K2 = 0x9E3779B97F4A7C15, 0xD1B54A32D192ED03, 0x8CB92BA72F3D8DD7
M64 = (1 << 64) - 1


def uniform(seed, index, draw):
    """The generator's float in [0, 1) for arrays of body indices."""
    with np.errstate(over="ignore"):
        i = np.asarray(index, dtype=np.uint64)
        z = (np.uint64(seed * K0 & M64) + (i + np.uint64(1)) * np.uint64(K1) +
             np.uint64((draw + 1) * K2 & M64))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def _sim(n):
    sim = BarnesHut(n, np.array([-1, -1, -1, 1, 1, 1], np.float32), abi.units(G=1.0))
    return sim


def test_box_matches_restated_generator(gbh_lib):
    n, seed = 50000, 12345
    ranges = [(-2, 3), (0, 1), (-1, -0.5), (-0.1, 0.1), (0, 0), (1, 2), (1e-6, 1e-3), (0.5, 4)]
    sim = _sim(n)
    sim.generate_bodies(abi.ic_params(abi.IC_BOX, ranges=ranges), seed=seed)
    got = sim.read_bodies()
    idx = np.arange(n)
    cols = []
    for k, (lo, hi) in enumerate(ranges):
        lo32, hi32 = np.float32(lo), np.float32(hi)
        cols.append(uniform(seed, idx, k) * (hi32 - lo32) + lo32)
    want = np.stack(cols, axis=1).astype(np.float32)
    flat = np.concatenate([got["pos_mass"][:, :3], got["vel_density"][:, :3], got["pos_mass"][:, 3:],
                           got["vel_density"][:, 3:]], axis=1)
    assert np.array_equal(flat.view(np.uint32), want.view(np.uint32))


def test_chunks_equal_one_shot(gbh_lib):
    n = 70001
    p = abi.ic_params(abi.IC_PLUMMER, scale=1.0, total_mass=1.0)
    a, b = _sim(n), _sim(n)
    a.generate_bodies(p, seed=7)
    b.generate_bodies(p, seed=7, count=30000, offset=0)
    b.generate_bodies(p, seed=7, count=n - 30000, offset=30000)
    # the equal-mass split uses the count of the call: compare positions and velocities
    ga, gb = a.read_bodies(), b.read_bodies()
    assert np.array_equal(ga["pos_mass"][:, :3], gb["pos_mass"][:, :3])
    assert np.array_equal(ga["vel_density"], gb["vel_density"])


def test_plummer_half_mass_radius_and_virial_ratio(gbh_lib):
    n = 8192
    sim = _sim(n)
    sim.generate_bodies(abi.ic_params(abi.IC_PLUMMER, scale=2.0, total_mass=3.0, G=1.0), seed=3)
    b = sim.read_bodies()
    x = b["pos_mass"][:, :3].astype(np.float64)
    v = b["vel_density"][:, :3].astype(np.float64)
    m = b["pos_mass"][:, 3].astype(np.float64)
    assert np.allclose(m, 3.0 / n)
    r = np.linalg.norm(x, axis=1)
    # half-mass radius of a Plummer sphere: a / sqrt(2^(2/3) - 1) = 1.3048 a
    assert np.median(r) == pytest.approx(2.0 * 1.3048, rel=0.04)
    kin = 0.5 * (m * (v * v).sum(1)).sum()
    pot = 0.0
    for s in range(0, n, 1024):
        d = np.linalg.norm(x[s:s + 1024, None, :] - x[None, :, :], axis=2)
        w = m[s:s + 1024, None] * m[None, :] / np.where(d > 0, d, np.inf)
        pot -= 0.5 * w.sum()
    assert 2 * kin / abs(pot) == pytest.approx(1.0, abs=0.1)


def test_disk_in_plane_orbits_and_centre_body_last(gbh_lib):
    n = 20001
    phi = 0.4
    p = abi.ic_params(abi.IC_DISK, ranges=[(1.0, 5.0)] + [(0, 0)] * 5 + [(1e-6, 2e-6), (1.0, 1.0)],
                      center=(1.0, 2.0, 3.0), velocity=(0.1, 0.0, 0.0), G=1.0, phi=phi, center_mass=10.0,
                      center_density=2.0, adherence=1.0, orbital_factor=1.0, flags=abi.IC_ORBITAL)
    sim = _sim(n)
    sim.generate_bodies(p, seed=5)
    b = sim.read_bodies()
    c = np.array([1.0, 2.0, 3.0])
    assert np.allclose(b["pos_mass"][-1], [1.0, 2.0, 3.0, 10.0])
    x = b["pos_mass"][:-1, :3].astype(np.float64) - c
    v = b["vel_density"][:-1, :3].astype(np.float64) - np.array([0.1, 0.0, 0.0])
    normal = np.array([0.0, np.sin(phi), np.cos(phi)])
    r = np.linalg.norm(x, axis=1)
    assert r.min() >= 1.0 - 1e-5 and r.max() <= 5.0 + 1e-5
    assert np.abs(x @ normal).max() < 1e-5 * r.max()  # adherence 1: in the plane
    assert np.abs((x * v).sum(1)).max() < 1e-4 * (r * np.linalg.norm(v, axis=1)).max()  # tangential
    approx = (2e-6 + 1e-6) / 2 * (n - 1) * (r / 5.0) ** 3.0
    np.testing.assert_allclose(np.linalg.norm(v, axis=1), np.sqrt((10.0 + approx) / r), rtol=1e-4)
    m = b["pos_mass"][:-1, 3]
    assert m.min() >= 1e-6 and m.max() <= 2e-6


def test_clusters_around_their_centres(gbh_lib):
    n, k, seed = 100000, 16, 9
    p = abi.ic_params(abi.IC_CLUSTERS, ranges=[(0, 0)] * 6 + [(1e-9, 1e-6), (1, 1)], scale=10.0, clusters=k,
                      sigma_lo=0.01, sigma_hi=0.1, density=3.0)
    sim = _sim(n)
    sim.generate_bodies(p, seed=seed)
    b = sim.read_bodies()
    which = np.minimum((uniform(seed, np.arange(n), 0) * np.float32(k)).astype(np.int64), k - 1)
    cseed = (seed + 0x632BE59BD9B4E019) & M64
    centres = np.stack([(2 * uniform(cseed, np.arange(k), d).astype(np.float64) - 1) * 10.0 for d in range(3)], 1)
    sig = np.exp(np.log(0.01) + uniform(cseed, np.arange(k), 3).astype(np.float64) * (np.log(0.1) - np.log(0.01)))
    d = np.linalg.norm(b["pos_mass"][:, :3] - centres[which], axis=1)
    assert np.all(d < 7.0 * sig[which])
    m = b["pos_mass"][:, 3]
    assert m.min() >= 1e-9 * (1 - 1e-5) and m.max() <= 1e-6 * (1 + 1e-5)
    assert np.all(b["vel_density"][:, 3] == 3.0)
    # the m^-2 law: a quarter of the bodies below 4/3 of the lower mass
    assert np.mean(m < 4e-9 / 3) == pytest.approx(0.25, abs=0.01)


def test_generated_state_steps(gbh_lib):
    n = 65536
    sim = BarnesHut(n, np.array([-20, -20, -20, 20, 20, 20], np.float32), abi.units(G=1.0))
    sim.generate_bodies(abi.ic_params(abi.IC_PLUMMER, scale=1.0, total_mass=1.0), seed=1)
    sim.init()
    sim.step(abi.step_params(theta=0.5, softening=1e-4), count=3)
    sim.synchronize()
    assert sim.read_stats().error_word == 0 and sim.read_stats().alive == n
