"""The precision form (GBH_PRECISION_COMPENSATED): FP64 drift, walk offsets
from the FP32 position plus its FP32 residual with compensated near-field
sums, the FP64 direct sum and the FP64 diagnostics, against FP64 numpy."""
import numpy as np
import pytest

from gravity_gb300 import BarnesHut, abi, accuracy, ic

pytestmark = pytest.mark.gpu


def _sim(bodies, bounds=None):
    sim = BarnesHut(len(bodies), bounds if bounds is not None else ic.exact_bounds(bodies), abi.units(G=1.0))
    sim.upload_bodies(bodies)
    sim.init()
    return sim


def test_fp64_drift_keeps_sub_ulp_motion(gbh_lib):
    # bodies near x = 100 (FP32 ulp 7.6e-6) moving 1e-6 per step: the FP32
    # drift rounds every step's move away, the FP64 drift accumulates it
    n = 4096
    rng = np.random.default_rng(0)
    b = np.zeros(n, dtype=abi.BODY_DTYPE)
    pos = 100.0 + rng.uniform(-0.5, 0.5, (n, 3))
    b["pos_mass"][:, :3] = pos
    b["pos_mass"][:, 3] = 1e-12  # negligible gravity
    b["vel_density"][:, 0] = 1e-3
    b["vel_density"][:, 3] = 1.0
    steps, dt = 50, 1e-3
    p32 = abi.step_params(dt=dt, theta=0.5, softening=1e-4)
    p64 = abi.step_params(dt=dt, theta=0.5, softening=1e-4, precision=abi.PRECISION_COMPENSATED)
    s32, s64 = _sim(b), _sim(b)
    x0 = s64.read_bodies()["pos_mass"][:, 0].astype(np.float64)
    s32.step(p32, count=steps)
    s64.step(p64, count=steps)
    s32.synchronize()
    s64.synchronize()
    moved32 = s32.read_bodies()["pos_mass"][:, 0].astype(np.float64) - x0
    x64 = s64.read_positions_fp64()
    moved64 = x64[:, 0] - x0
    want = steps * 1e-3 * dt
    assert np.all(np.abs(moved32) < 1e-9)  # FP32: no motion at all
    np.testing.assert_allclose(moved64, want, rtol=1e-6)
    # the body buffer holds the FP32 rounding of the FP64 positions
    assert np.array_equal(s64.read_bodies()["pos_mass"][:, :3], x64.astype(np.float32))


@pytest.mark.parametrize("mac", [abi.MAC_PLAIN, abi.MAC_GROUP])
def test_compensated_walk_beats_fp32_against_fp64_direct_sum(gbh_lib, mac):
    # a compact cluster far from the origin, with FP64 positions whose FP32
    # rounding (ulp 7.6e-6 at 100) is comparable to the softening length
    n = 32768
    b = ic.plummer(n, seed=4)
    rng = np.random.default_rng(5)
    x = 100.0 + 0.002 * b["pos_mass"][:, :3].astype(np.float64) + rng.uniform(-4e-6, 4e-6, (n, 3))
    bounds = np.concatenate([x.min(0) - 1e-3, x.max(0) + 1e-3]).astype(np.float32)
    sim = _sim(b, bounds)
    sim.write_positions_fp64(x)
    soft = (4e-6) ** 2
    kw = dict(theta=0.05, softening=soft, mac=mac)
    p64 = abi.step_params(precision=abi.PRECISION_COMPENSATED, **kw)
    p32 = abi.step_params(**kw)
    sample = accuracy.sample_bodies(np.arange(n, dtype=np.uint32), 1024, seed=1)
    ref = sim.direct_sum(p64, sample)  # FP64 terms from the FP64 positions
    a64 = sim.evaluate_walk(p64)[sample].astype(np.float64)
    assert sim.read_stats().error_word == 0
    e64 = np.linalg.norm(a64 - ref, axis=1) / np.linalg.norm(ref, axis=1)
    # the FP32 form sees the rounded positions (the FP64 copy is no longer current after it)
    a32 = sim.evaluate_walk(p32)[sample].astype(np.float64)
    e32 = np.linalg.norm(a32 - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert np.median(e64) < 0.3 * np.median(e32), (np.median(e64), np.median(e32))
    assert np.percentile(e64, 99) < np.percentile(e32, 99)


def test_diagnostics_match_numpy_fp64(gbh_lib):
    n = 4096
    b = ic.plummer(n, seed=6)
    sim = _sim(b)
    p = abi.step_params(theta=0.2, softening=1e-4, precision=abi.PRECISION_COMPENSATED)
    d = sim.diagnostics(p)
    assert d["live_bodies"] == n and d["potential_valid"] == 1 and d["positions_fp64"] == 1
    m = b["pos_mass"][:, 3].astype(np.float64)
    x = b["pos_mass"][:, :3].astype(np.float64)
    v = b["vel_density"][:, :3].astype(np.float64)
    assert d["mass"] == pytest.approx(m.sum(), rel=1e-12)
    np.testing.assert_allclose(d["momentum"], (m[:, None] * v).sum(0), rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(d["centre_of_mass"], (m[:, None] * x).sum(0) / m.sum(), rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(d["angular_momentum"], (m[:, None] * np.cross(x, v)).sum(0), rtol=1e-9, atol=1e-12)
    assert d["kinetic_energy"] == pytest.approx(0.5 * (m * (v * v).sum(1)).sum(), rel=1e-9)
    # potential energy: the tree walk's against the exact pair sum
    r = x[:, None, :] - x[None, :, :]
    inv = 1.0 / np.sqrt((r * r).sum(-1) + 1e-4)
    np.fill_diagonal(inv, 0.0)
    w_exact = -0.5 * (m[:, None] * m[None, :] * inv).sum()
    assert d["potential_energy"] == pytest.approx(w_exact, rel=2e-3)
    # a step advances the state: its potential belongs to the previous positions
    sim.step(p)
    sim.synchronize()
    assert sim.diagnostics()["potential_valid"] == 0


def test_precision_form_runs_with_learned_walk_and_rejects_merges(gbh_lib):
    bodies = ic.plummer(16384, seed=7)
    sim = _sim(bodies)
    rng = np.random.default_rng(0)
    sim.mac_set_weights(rng.normal(0, 0.1, abi.MAC_NUM_PARAMS).astype(np.float32))
    p = abi.step_params(theta=0.5, softening=1e-4, mac=abi.MAC_LEARNED, mac_tolerance=-2.0,
                        precision=abi.PRECISION_COMPENSATED)
    sim.step(p, count=3)
    sim.synchronize()
    assert sim.read_stats().error_word == 0
    assert np.all(np.isfinite(sim.read_positions_fp64()))
    with pytest.raises(Exception):
        sim.step(abi.step_params(mode=abi.MODE_MERGE, precision=abi.PRECISION_COMPENSATED))
