"""Host helpers of the view and initial-condition parameter structs (no GPU)."""
import ctypes as C

import numpy as np
import pytest

from gravity_gb300 import abi


def test_look_at_maps_eye_to_origin_and_target_down_minus_z():
    eye, target = np.array([3.0, 4.0, 12.0]), np.array([0.0, 0.0, 0.0])
    m = abi.look_at(eye, target).astype(np.float64)
    assert np.allclose(m @ np.r_[eye, 1.0], [0, 0, 0, 1], atol=1e-5)
    t = m @ np.r_[target, 1.0]
    assert np.allclose(t[:2], 0, atol=1e-5) and t[2] == pytest.approx(-13.0, rel=1e-6)
    assert np.allclose(m[:3, :3] @ m[:3, :3].T, np.eye(3), atol=1e-6)  # a rotation


def test_perspective_maps_near_and_far_planes():
    fov, aspect, near, far = np.radians(60.0), 1.5, 0.1, 100.0
    p = abi.perspective(fov, aspect, near, far).astype(np.float64)
    for z, ndc in ((-near, -1.0), (-far, 1.0)):
        c = p @ np.array([0.0, 0.0, z, 1.0])
        assert c[2] / c[3] == pytest.approx(ndc, abs=1e-5)
    # a point on the top edge of the view at depth 10
    y = 10.0 * np.tan(0.5 * fov)
    c = p @ np.array([0.0, y, -10.0, 1.0])
    assert c[1] / c[3] == pytest.approx(1.0, rel=1e-5)


def test_view_stores_matrices_column_major_and_theta_in_ndc():
    mv = np.arange(16, dtype=np.float32).reshape(4, 4)
    v = abi.view(mv, np.eye(4), 1.0, 2.0, glow_theta_px=16.0, height=1080, region_depths=(3, 9))
    assert list(v.model_view)[:4] == [0.0, 4.0, 8.0, 12.0]  # first column
    assert v.glow_theta_ndc == pytest.approx(2 * 16 / 1080, rel=1e-6)
    assert (v.region_min_depth, v.region_max_depth) == (3, 9)
    assert v.relative_to == 0xFFFFFFFF and C.sizeof(v) == 176


def test_ic_params_ranges_and_fields():
    p = abi.ic_params(abi.IC_DISK, ranges=[(1.0, 5.0)] + [(0.0, 0.0)] * 5 + [(1e-6, 2e-6), (1.0, 3.0)],
                      center=(1.0, 2.0, 3.0), phi=0.5, flags=abi.IC_ORBITAL | abi.IC_CCW)
    assert p.kind == abi.IC_DISK and p.flags == 3
    assert (p.lo[0], p.hi[0]) == (1.0, 5.0) and p.hi[7] == 3.0
    assert list(p.center) == [1.0, 2.0, 3.0] and p.phi == pytest.approx(0.5)
    assert p.G == 1.0 and p.density == 1.0  # defaults
    with pytest.raises(TypeError):
        abi.ic_params(abi.IC_BOX, no_such_field=1.0)  # a misspelt field is an error, not ignored
