"""Replays a golden fixture (tests/golden/*.npz, produced by the reference's own
kernels) on an implementation with the stage API and compares the outputs."""
from __future__ import annotations

import glob
import os

import numpy as np

from gravity_gb300 import abi

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PARAM_FIELDS = ["dt", "theta", "softening", "elasticity", "restitution", "merging_collision_or_neither",
                "static_or_dynamic", "wrap_around"]


def same_bits(a, b) -> bool:
    """Bitwise equality of float arrays, with every NaN equal to every NaN
    (CUDA produces the canonical NaN, x86 its default NaN)."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    both_nan = np.isnan(a) & np.isnan(b)
    return bool(np.all((a.view(np.uint32) == b.view(np.uint32)) | both_nan))


def fixtures():
    """The small fixtures (inputs and outputs stored whole)."""
    return sorted(p for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))
                  if not os.path.basename(p).startswith(("large_", "view_")))


def large_fixtures():
    """The large fixtures (generated inputs, digests of the outputs)."""
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, "large_*.npz")))


def params_of(z) -> abi.StepParams:
    v = z["params"]
    p = abi.step_params()
    for f, x in zip(PARAM_FIELDS, v):
        setattr(p, f, type(getattr(p, f))(x))
    return p


def replay(path, make, exact_walk: bool, ordered_tasks: bool):
    """make(n, bounds, units) -> implementation.  exact_walk: bodies after the
    walk must be bit-identical (CPU oracle); otherwise within 1e-5."""
    z = np.load(path)
    bodies = z["bodies"]
    n = len(bodies)
    p = params_of(z)
    x = make(n, z["bounds"], abi.units(G=1.0))
    x.upload_bodies(bodies)
    x.init()
    for k in range(int(z["steps"])):
        pre = f"s{k}_"
        x.stage_reset(p)
        x.stage_prepare(p)
        s = x.read_sim_values()
        assert s.num_bodies == int(z[pre + "prep_num_bodies"]), path
        b = np.array(list(s.bounds_min) + list(s.bounds_max), np.float32)
        assert np.array_equal(b, z[pre + "prep_bounds"]), (path, b, z[pre + "prep_bounds"])
        assert np.array_equal(x.read_index(), z[pre + "prep_index"]), path
        nl = s.num_bodies
        assert np.array_equal(x.read_morton()[:nl], z[pre + "prep_morton"]), path
        x.stage_sort()
        x.stage_build()
        x.stage_fill()
        x.stage_walk(p)
        tasks = x.read_merge_tasks()
        gold = z[pre + "tasks"]
        if ordered_tasks:
            assert np.array_equal(tasks, gold), path
        else:
            assert set(map(tuple, tasks.tolist())) == set(map(tuple, gold.tolist())), path
        x.stage_merge(p)
        x.stage_swap()
        assert np.array_equal(x.read_index()[:nl], z[pre + "sorted_index"]), path
        assert np.array_equal(x.read_morton()[:nl], z[pre + "sorted_morton"]), path
        gi, gl = z[pre + "internal"], z[pre + "leaf"]
        xi, xl = x.read_internal_nodes()[: len(gi)], x.read_leaf_nodes()[:nl]
        for f in ("child_a", "child_b", "parent_id", "bodies_contained", "node_depth", "ready_children"):
            assert np.array_equal(xi[f], gi[f]), (path, f)
            assert np.array_equal(xl[f], gl[f]), (path, f)
        for f in ("com_mass", "aabb"):
            assert same_bits(xi[f], gi[f]), (path, f)
            assert same_bits(xl[f], gl[f]), (path, f)
        np.testing.assert_allclose(xi["avg_color"], gi["avg_color"], rtol=1e-5, atol=1e-6, equal_nan=True)
        after = x.read_bodies()
        gb = z[pre + "bodies_after"]
        if exact_walk:
            assert same_bits(after.view(np.float32), gb.view(np.float32)), path
            assert x.read_sim_values().uint_debug[0] == int(z[pre + "uint_debug0"]), path
        else:
            assert np.array_equal(after["pos_mass"][:, 3] == 0, gb["pos_mass"][:, 3] == 0), path
            np.testing.assert_allclose(after["pos_mass"], gb["pos_mass"], rtol=1e-5, atol=1e-6, equal_nan=True)
            np.testing.assert_allclose(after["vel_density"], gb["vel_density"], rtol=1e-4, atol=1e-5, equal_nan=True)
            # later steps start from the reference's state so that each step is compared on equal inputs
            x.upload_bodies(gb)
        assert x.read_sim_values().out_of_bounds == int(z[pre + "out_of_bounds"]), path
    return True


def replay_large(path, make, exact_walk: bool):
    """One step of a large fixture: inputs regenerated (digest checked), every
    exact output compared by digest; bodies after the step bit-identical
    (exact_walk) or, on every 16th body, within 1e-5."""
    from tests.golden import large_inputs as L

    z = np.load(path)
    kind, n, seed = str(z["kind"]), int(z["n"]), int(z["seed"])
    bodies = L.make(kind, n, seed)
    assert L.digest(bodies) == str(z["input_sha256"]), (path, "regenerated inputs differ")
    p = params_of(z)
    x = make(n, z["bounds"], abi.units(G=1.0))
    x.upload_bodies(bodies)
    x.init()
    x.stage_reset(p)
    x.stage_prepare(p)
    s = x.read_sim_values()
    nl = s.num_bodies
    assert nl == int(z["prep_num_bodies"]), path
    assert np.array_equal(np.array(list(s.bounds_min) + list(s.bounds_max), np.float32), z["prep_bounds"]), path
    assert L.digest(x.read_index()) == str(z["prep_index"]), path
    assert L.digest(x.read_morton()[:nl]) == str(z["prep_morton"]), path
    x.stage_sort()
    x.stage_build()
    x.stage_fill()
    x.stage_walk(p)
    tasks = x.read_merge_tasks()
    assert len(tasks) == int(z["task_count"]), path
    assert L.task_digest(tasks) == str(z["tasks"]), path
    x.stage_merge(p)
    x.stage_swap()
    assert L.digest(x.read_index()[:nl]) == str(z["sorted_index"]), path
    assert L.digest(x.read_morton()[:nl]) == str(z["sorted_morton"]), path
    for f, d in L.node_digests(x.read_internal_nodes()[: max(nl - 1, 1)]).items():
        assert d == str(z[f"internal_{f}"]), (path, "internal", f)
    for f, d in L.node_digests(x.read_leaf_nodes()[:nl]).items():
        assert d == str(z[f"leaf_{f}"]), (path, "leaf", f)
    after = x.read_bodies()
    assert L.digest((after["pos_mass"][:, 3] == 0).astype(np.uint8)) == str(z["dead_after"]), path
    if exact_walk:
        assert L.digest(after.view(np.float32)) == str(z["bodies_after"]), path
        assert x.read_sim_values().uint_debug[0] == int(z["uint_debug0"]), path
    else:
        gb = z["bodies_sample"]
        mine = after[::16]
        np.testing.assert_allclose(mine["pos_mass"], gb["pos_mass"], rtol=1e-5, atol=1e-6, equal_nan=True)
        np.testing.assert_allclose(mine["vel_density"], gb["vel_density"], rtol=1e-4, atol=1e-5, equal_nan=True)
    assert x.read_sim_values().out_of_bounds == int(z["out_of_bounds"]), path
    return True


# ---- node selection against the reference's vertex shaders -------------------
VIEW_FIXTURE = os.path.join(GOLDEN_DIR, "view_select.npz")
_BOX = np.float32(1.5)
_MAPPING = np.array([[-1, -1], [-1, 1], [1, -1], [1, 1]], np.float32) * _BOX  # nodeglow.vert vertices 0-3


def view_fixture():
    z = np.load(VIEW_FIXTURE)
    views = []
    k = 0
    while f"v{k}_view" in z:
        v = abi.View.from_buffer_copy(z[f"v{k}_view"].tobytes())
        views.append((v, z[f"v{k}_mvp"]))
        k += 1
    return z, views


def tree_of_view_fixture(make):
    """The fixture's tree (reset, compaction, sort, build, fill of its bodies)
    on an implementation with the stage API; returns it and its live count."""
    z = np.load(VIEW_FIXTURE)
    p = params_of(z)
    x = make(len(z["bodies"]), z["bounds"], abi.units(G=1.0))
    x.upload_bodies(z["bodies"])
    x.init()
    x.stage_reset(p)
    x.stage_prepare(p)
    x.stage_sort()
    x.stage_build()
    x.stage_fill()
    return x, x.read_sim_values().num_bodies


def _f32(x):
    return np.float32(x)


def _mat4_vec4(m16, v):
    """uMVP * v with the column terms added in column order, in FP32."""
    M = np.asarray(m16, np.float32).reshape(4, 4)  # [column][row]
    out = np.zeros(4, np.float32)
    for i in range(4):
        s = _f32(M[0, i] * v[0])
        s = _f32(s + _f32(M[1, i] * v[1]))
        s = _f32(s + _f32(M[2, i] * v[2]))
        s = _f32(s + _f32(M[3, i] * v[3]))
        out[i] = s
    return out


def check_glow_against_shader(records, z, k):
    """Records of gbh_select_glow_nodes (any order) against the shader's
    outputs for view k: the same nodes; vIntensity, vColor, vCenterView and
    the NDC scales bit for bit; gl_Position of the four vertices rebuilt from
    the record in the shader's operation order, bit for bit."""
    r = np.sort(records, order="node")
    assert np.array_equal(r["node"], z[f"v{k}_glow_nodes"]), "glow selection differs"
    o = z[f"v{k}_glow_outputs"]
    assert same_bits(r["intensity"], o[:, 0])
    assert same_bits(r["color"][:, :3], o[:, 1:4])
    assert same_bits(r["center_view"], o[:, 4:7])
    assert same_bits(r["ndc_scale"], o[:, 7:9])
    pos = z[f"v{k}_glow_position"]
    for i in range(len(r)):
        c = r["center_clip"][i].astype(np.float32)
        scale = r["ndc_scale"][i].astype(np.float32)
        for vid in range(4):
            off = (_MAPPING[vid] * scale) * c[3]
            want = np.array([c[0] + off[0], c[1] + off[1], c[2], c[3]], np.float32)
            assert same_bits(want, pos[i, vid]), (k, int(r["node"][i]), vid)


def check_regions_against_shader(records, z, k, mvp):
    """Records of gbh_select_regions against regions.vert for view k: the same
    nodes and depths; gl_Position at two opposite unit-cube corners rebuilt
    from the record's centre and size (center + aPos * size, then uMVP),
    bit for bit."""
    r = np.sort(records, order="node")
    assert np.array_equal(r["node"], z[f"v{k}_region_nodes"]), "region selection differs"
    assert np.array_equal(r["depth"], z[f"v{k}_region_depth"])
    pos = z[f"v{k}_region_position"]
    for i in range(len(r)):
        cen = r["center"][i].astype(np.float32)
        size = r["size"][i].astype(np.float32)
        for j, a in enumerate((np.float32(-0.5), np.float32(0.5))):
            w = cen + a * size
            got = _mat4_vec4(mvp, np.array([w[0], w[1], w[2], 1.0], np.float32))
            assert same_bits(got, pos[i, j]), (k, int(r["node"][i]), j)
