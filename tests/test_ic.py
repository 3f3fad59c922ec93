"""Seeded initial conditions: deterministic, the requested sizes and shapes."""
import numpy as np

from gravity_gb300 import abi, ic


def test_plummer_deterministic_and_centred():
    a = ic.plummer(20000, seed=0)
    b = ic.plummer(20000, seed=0)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert a.dtype == abi.BODY_DTYPE
    p = a["pos_mass"][:, :3].astype(np.float64)
    assert np.allclose(a["pos_mass"][:, 3].sum(), 1.0, rtol=1e-4)
    r = np.linalg.norm(p, axis=1)
    # half-mass radius of a Plummer sphere: a / sqrt(2^(2/3) - 1) = 1.305 a
    assert abs(np.median(r) - 1.305) < 0.05
    # virial ratio of the DF velocities: 2T / |W| ~ 1, with W = -3 pi M^2 / (32 a)
    T = 0.5 * np.sum(a["pos_mass"][:, 3] * np.sum(a["vel_density"][:, :3].astype(np.float64) ** 2, axis=1))
    W = -3 * np.pi / 32
    assert abs(2 * T / abs(W) - 1.0) < 0.1


def test_uniform_merge_radii():
    b = ic.uniform_merge(10000, seed=1)
    m = b["pos_mass"][:, 3].astype(np.float64)
    assert m.min() >= 1e-6 * 0.999 and m.max() <= 1e-3 * 1.001
    r = 0.6203504909 * (m / b["vel_density"][:, 3]) ** (1 / 3)
    np.testing.assert_allclose(r, 0.002 * (m / 1e-3) ** (1 / 3), rtol=1e-5)
    assert np.all(np.abs(b["pos_mass"][:, :3]) <= 1)


def test_mixture_and_clusters_and_galaxies():
    m = ic.plummer_uniform(10000, seed=3)
    assert len(m) == 10000 and np.allclose(m["pos_mass"][:, 3], 1e-4)
    c = ic.cluster_mixture(20000, seed=4, clusters=16)
    assert c["pos_mass"][:, 3].min() >= 1e-9 * 0.999 and c["pos_mass"][:, 3].max() <= 1e-6 * 1.001
    g = ic.galaxy_pair(5000, seed=2)
    assert len(g) == 10000
    x = g["pos_mass"][:, 0]
    assert (x < 0).sum() > 4000 and (x > 0).sum() > 4000
