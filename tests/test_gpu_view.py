"""Headless level-of-detail node selection on the GPU (gbh_select_glow_nodes,
gbh_select_regions) against the oracle's restatement of nodeglow.vert and
regions.vert, on the tree of a real step.  Both compute in FP32 with one
rounding per operation in the same order, so the records must be identical
(sorted by node); the tolerance is zero."""
import numpy as np
import pytest

from gravity_gb300 import BarnesHut, abi, ic

pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.oracle")


@pytest.fixture(scope="module")
def stepped():
    n = 65536
    b = ic.plummer(n, seed=11)
    sim = BarnesHut(n, ic.exact_bounds(b), abi.units(G=1.0))
    sim.upload_bodies(b)
    sim.init()
    sim.step(abi.step_params(theta=0.5, softening=1e-4))
    sim.synchronize()
    live = sim.read_stats().alive
    nodes = sim.read_internal_nodes(live - 1)
    bodies = sim.read_bodies()
    return sim, nodes, bodies


def _views():
    fov, aspect = np.radians(50.0), 16.0 / 9.0
    proj = abi.perspective(fov, aspect, 0.01, 1e5)
    out = []
    for eye, rel, scale, depths in [((0, 0, 60), 0xFFFFFFFF, 10.0, (2, 6)),
                                    ((30, 20, 15), 0xFFFFFFFF, 10.0, (0, 3)),
                                    ((5, -4, 8), 7, 1.0, (4, 30))]:
        out.append(abi.view(abi.look_at(eye, (0, 0, 0)), proj, fov, aspect, camera_scale=scale, relative_to=rel,
                            glow_max_depth=12, glow_intensity=0.05, region_depths=depths))
    return out


@pytest.mark.parametrize("k", range(3))
def test_glow_selection_matches_oracle(gbh_lib, stepped, k):
    sim, nodes, bodies = stepped
    v = _views()[k]
    got, sel = sim.select_glow_nodes(v)
    want, sel_o = O.select_glow_nodes(nodes, bodies, v)
    assert sel == sel_o and sel > 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("k", range(3))
def test_region_selection_matches_oracle(gbh_lib, stepped, k):
    sim, nodes, bodies = stepped
    v = _views()[k]
    got, sel = sim.select_regions(v)
    want, sel_o = O.select_regions(nodes, bodies, v)
    assert sel == sel_o and sel > 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_selection_capacity_keeps_the_count(gbh_lib, stepped):
    sim, nodes, bodies = stepped
    v = _views()[0]
    full, sel = sim.select_regions(v)
    part, sel2 = sim.select_regions(v, capacity=16)
    assert sel2 == sel > 16 and len(part) == 16
    assert set(part["node"].tolist()) <= set(full["node"].tolist())
    # a count-only query writes nothing
    none, sel3 = sim.select_regions(v, capacity=0)
    assert sel3 == sel and len(none) == 0


def test_selection_matches_reference_shaders(gbh_lib):
    # the GPU's tree of the fixture's bodies (bit-exact with the reference's)
    # and its selection against the outputs of the reference's own vertex
    # shaders (tests/golden/view_select.npz), bit for bit
    from .golden_check import check_glow_against_shader, check_regions_against_shader, tree_of_view_fixture, \
        view_fixture

    z, views = view_fixture()
    sim, n = tree_of_view_fixture(BarnesHut)
    for k, (v, mvp) in enumerate(views):
        g, sel = sim.select_glow_nodes(v)
        assert sel > 0
        check_glow_against_shader(g, z, k)
        r, sel = sim.select_regions(v)
        assert sel > 0
        check_regions_against_shader(r, z, k, mvp)
