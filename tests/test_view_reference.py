"""The oracle's node selection (orc_select_glow_nodes, orc_select_regions)
against the reference's own node-glow and region vertex shaders
(src/main/resources/shaders/render/nodeglow/nodeglow.vert:46-148,
render/regions/regions.vert:19-43), compiled as C++ by
oracle/ref_glsl/ref_render.cpp.

The fixture tests/golden/view_select.npz holds the shaders' outputs over the
reference's tree of a 2,048-body Plummer sphere for three views
(tests/golden/make_golden.py); the oracle's tree of the same bodies is bit-exact
with the reference's, and its selection must reproduce the shader outputs bit
for bit.  Where the reference sources are mounted, the shaders also run live on
a second tree."""
import numpy as np
import pytest

from gravity_gb300 import abi, ic

from .golden_check import check_glow_against_shader, check_regions_against_shader, tree_of_view_fixture, view_fixture


def test_oracle_selection_matches_reference_shaders_golden(oracle_mod):
    z, views = view_fixture()
    x, n = tree_of_view_fixture(oracle_mod.OracleBarnesHut)
    nodes, bodies = x.read_internal_nodes()[: n - 1], x.read_bodies()
    for k, (v, mvp) in enumerate(views):
        g, sel = oracle_mod.select_glow_nodes(nodes, bodies, v)
        assert sel > 0
        check_glow_against_shader(g, z, k)
        r, sel = oracle_mod.select_regions(nodes, bodies, v)
        assert sel > 0
        check_regions_against_shader(r, z, k, mvp)


def test_oracle_selection_matches_reference_shaders_live(oracle_mod):
    from oracle import ref_harness as R

    if not R.available():
        pytest.skip("reference sources not mounted")
    R.build_if_available()
    n = 3000
    b = ic.plummer(n, seed=44)
    b["pos_mass"][:, :3] *= 2.0
    o = oracle_mod.OracleBarnesHut(n, ic.exact_bounds(b), abi.units(G=1.0))
    o.upload_bodies(b)
    o.init()
    p = abi.step_params(theta=0.5, softening=1e-4)
    o.step(p)
    o.stage_reset(p)
    o.stage_prepare(p)
    o.stage_sort()
    o.stage_build()
    o.stage_fill()
    nodes, bodies = o.read_internal_nodes()[: n - 1], o.read_bodies()
    fov, aspect = np.radians(40.0), 1.5
    proj = abi.perspective(fov, aspect, 0.01, 1e5)
    for eye, rel in (((0, 0, 30), 0xFFFFFFFF), ((12, -9, 4), 3)):
        mv = abi.look_at(eye, (0, 0, 0))
        v = abi.view(mv, proj, fov, aspect, camera_scale=5.0, relative_to=rel, glow_max_depth=10,
                     glow_intensity=0.02, region_depths=(1, 9))
        mvp = (np.asarray(proj, np.float64) @ np.asarray(mv, np.float64)).astype(np.float32).T.reshape(-1)
        glow, reg = R.render_instances(nodes, bodies, n, v, mvp)
        gsel = np.nonzero(glow[:, 0, 6] != 0)[0]
        culled = (reg[:, 0, 0] == 2) & (reg[:, 0, 1] == 2) & (reg[:, 0, 2] == 2) & (reg[:, 0, 3] == 1)
        rsel = np.nonzero(~culled[: n - 1])[0]
        z = {"v0_glow_nodes": gsel.astype(np.uint32), "v0_glow_position": glow[gsel][:, :, 0:4],
             "v0_glow_outputs": glow[gsel][:, 0, 6:15], "v0_region_nodes": rsel.astype(np.uint32),
             "v0_region_position": reg[rsel][:, :, 0:4], "v0_region_depth": reg[rsel][:, 0, 4].astype(np.uint32)}
        g, _ = oracle_mod.select_glow_nodes(nodes, bodies, v)
        check_glow_against_shader(g, z, 0)
        r, _ = oracle_mod.select_regions(nodes, bodies, v)
        check_regions_against_shader(r, z, 0, mvp)
