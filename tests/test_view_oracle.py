"""The oracle's restatement of the render shaders' level-of-detail selection
(nodeglow.vert:46-150, regions.vert:19-45) on hand-built nodes: every cull
gate, and the drawn node's outputs against the shader formulas evaluated in
FP64 (the oracle computes in FP32)."""
import numpy as np
import pytest

from gravity_gb300 import abi

O = pytest.importorskip("oracle.oracle")

FOV = np.radians(60.0)
ASPECT = 16.0 / 9.0


def _node(lo, hi, com, mass, depth, bodies=10, color=(0.5, 0.25, 1.0)):
    n = np.zeros(1, dtype=abi.NODE_DTYPE)
    n["com_mass"][0] = [*com, mass]
    n["aabb"][0] = [*lo, *hi]
    n["node_depth"][0] = depth
    n["bodies_contained"][0] = bodies
    n["avg_color"][0] = [*color, 0.0]
    return n


def _view(**kw):
    mv = np.eye(4, dtype=np.float32)
    mv[2, 3] = -100.0  # camera at z = +100 looking down -z
    proj = abi.perspective(FOV, ASPECT, 0.1, 1e4)
    args = dict(camera_scale=1.0, glow_theta_px=16.0, height=1080, glow_max_depth=8, glow_intensity=0.003,
                region_depths=(2, 3))
    args.update(kw)
    return abi.view(mv, proj, FOV, ASPECT, **args), mv, proj


def _expected_glow(node, mv, proj, theta_ndc, intensity_scale):
    # nodeglow.vert in FP64
    lo, hi = node["aabb"][0][:3].astype(np.float64), node["aabb"][0][3:].astype(np.float64)
    longest = (hi - lo).max()
    com = node["com_mass"][0][:3].astype(np.float64)
    cv = mv.astype(np.float64) @ np.r_[com, 1.0]
    cam = max(-cv[2], 1e-6)
    th = np.tan(0.5 * np.float32(FOV))
    pe = longest / (cam * th)
    mn = theta_ndc * 0.04

    def ss(e0, e1, x):
        t = np.clip((x - e0) / (e1 - e0), 0, 1)
        return t * t * (3 - 2 * t)

    acc = (1 - ss(theta_ndc * 0.75, theta_ndc, pe)) * ss(mn, mn * 2.5, pe)
    raw = node["com_mass"][0][3] * (1e6 / cam ** 2) / max(pe * pe, 1e-8) * 2.5e-4 * acc * intensity_scale
    half = max(0.5 * longest * 1.1, mn * 0.5 * cam * th)
    ndc_y = half / (cam * th)
    return dict(center_view=cv[:3], center_clip=proj.astype(np.float64) @ cv, intensity=raw / (1 + raw),
                ndc_scale=[ndc_y / ASPECT, ndc_y])


def test_glow_draws_a_node_inside_the_band():
    v, mv, proj = _view()
    node = _node((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), (0.1, 0.0, 0.0), mass=10.0, depth=3)
    bodies = np.zeros(4, dtype=abi.BODY_DTYPE)
    rec, sel = O.select_glow_nodes(node, bodies, v)
    assert sel == 1 and rec["node"][0] == 0 and rec["depth"][0] == 3
    want = _expected_glow(node, mv, proj, 2.0 * 16.0 / 1080.0, 0.003)
    np.testing.assert_allclose(rec["center_view"][0], want["center_view"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(rec["center_clip"][0], want["center_clip"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(rec["intensity"][0], want["intensity"], rtol=1e-5)
    np.testing.assert_allclose(rec["ndc_scale"][0], want["ndc_scale"], rtol=1e-5)
    np.testing.assert_array_equal(rec["color"][0], np.float32([0.5, 0.25, 1.0]))


@pytest.mark.parametrize("case", ["too_coarse", "too_fine", "leaf_height", "too_tall", "empty_box", "massless",
                                  "no_bodies", "faint", "too_close"])
def test_glow_cull_gates(case):
    kw = {}
    lo, hi, com, mass, depth, nb = (-0.5,) * 3, (0.5,) * 3, (0.0,) * 3, 10.0, 3, 10
    if case == "too_coarse":
        lo, hi = (-1.0,) * 3, (1.0,) * 3  # projected 0.035 >= theta 0.0296: opened
    elif case == "too_fine":
        lo, hi = (-0.01,) * 3, (0.01,) * 3  # below 0.04 theta
    elif case == "leaf_height":
        depth = 0
    elif case == "too_tall":
        depth = 9
    elif case == "empty_box":
        lo, hi = (1.0,) * 3, (-1.0,) * 3
    elif case == "massless":
        mass = 0.0
    elif case == "no_bodies":
        nb = 0
    elif case == "faint":
        mass = 1e-12
    elif case == "too_close":
        kw["glow_activate_dist"] = 200.0
    v, _, _ = _view(**kw)
    rec, sel = O.select_glow_nodes(_node(lo, hi, com, mass, depth, nb), np.zeros(1, abi.BODY_DTYPE), v)
    assert sel == 0 and len(rec) == 0


def test_regions_depth_range_and_relative_location():
    nodes = np.concatenate([
        _node((0, 0, 0), (2, 4, 6), (1, 1, 1), 1.0, d) for d in (1, 2, 3, 4)
    ] + [_node((1, 1, 1), (0, 0, 0), (0, 0, 0), 1.0, 2)])  # empty box: culled
    bodies = np.zeros(3, dtype=abi.BODY_DTYPE)
    bodies["pos_mass"][2] = [1.0, 2.0, 3.0, 1.0]
    v, _, _ = _view(camera_scale=2.0, relative_to=2)
    rec, sel = O.select_regions(nodes, bodies, v)
    assert sel == 2 and list(rec["node"]) == [1, 2] and list(rec["depth"]) == [2, 3]
    # box relative to body 2, times the camera scale: min (-2,-4,-6), max (2,4,6)
    np.testing.assert_array_equal(rec["center"], np.zeros((2, 3), np.float32))
    np.testing.assert_array_equal(rec["size"], np.float32([[4, 8, 12]] * 2))
    # an index past the bodies means absolute coordinates
    v, _, _ = _view(camera_scale=2.0, relative_to=7)
    rec, _ = O.select_regions(nodes, bodies, v)
    np.testing.assert_array_equal(rec["center"][0], np.float32([2, 4, 6]))
