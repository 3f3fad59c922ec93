"""Parity at the benchmark sizes, through the C ABI.

The default bench workload (16,777,216 bodies: 70% Plummer + 30% uniform,
seed 3, the bench's own generator) runs stage by stage on the GPU and in the
CPU oracle.  At this size the sort runs 4,096 tiles per pass, so its
decoupled look-back walks long chains, and the tiled fill hands about 65,000
nodes across tiles to its top-tree pass; both must stay bit-exact:
  * compaction order, bounds and Morton keys;
  * the sort permutation (stable, ties in compaction order);
  * the tree topology and the fill's centre-of-mass, AABB and height words;
  * the plain walk's accelerations within 1e-5 median relative error (GLSL
    inversesqrt is rsqrtf on the GPU and 1/sqrtf in the oracle).
The step graph (in-order positions, one launch per step) must leave the same
state bit for bit as the eager stages at this size.

The merge workload (1,048,576 bodies uniform in [-1,1]^3, static box
[-2,2]^3, merges on) runs several consecutive steps; before each step the
oracle takes the GPU's state, so both start every step from the same bits,
and the merge tasks, the merged count, the pattern of live bodies and the
out-of-bounds count must be equal.
"""
import numpy as np
import pytest

from gravity_gb300 import BarnesHut, abi, ic

from .helpers import rel_err, sim_bounds

pytestmark = pytest.mark.gpu

N_C4 = 16777216
N_C2 = 1048576
CHUNK = 1 << 21


def _c4_params(**kw):
    return abi.step_params(dt=1e-3, theta=0.5, softening=0.005 ** 2, bounds=abi.BOUNDS_DYNAMIC, **kw)


@pytest.fixture(scope="module")
def c4_bodies():
    return ic.plummer_uniform(N_C4, seed=3)


def _equal_in_chunks(read_g, read_o, total, fields_exact, fields_bits, label):
    for off in range(0, total, CHUNK):
        cnt = min(CHUNK, total - off)
        a, b = read_g(cnt, off), read_o(cnt, off)
        for f in fields_exact:
            assert np.array_equal(a[f], b[f]), (label, f, off)
        for f in fields_bits:
            assert np.array_equal(a[f].view(np.uint32), b[f].view(np.uint32)), (label, f, off)


def test_c4_stages_bit_exact_and_walk(gbh_lib, oracle_mod, c4_bodies):
    n = N_C4
    bounds = ic.exact_bounds(c4_bodies)
    units = abi.units(G=1.0)
    g = BarnesHut(n, bounds, units)
    o = oracle_mod.OracleBarnesHut(n, bounds, units)
    for x in (g, o):
        x.upload_bodies(c4_bodies)
        x.init()
    p = _c4_params(flags=abi.FLAG_STORE_ACCEL)
    for x in (g, o):
        x.stage_reset(p)
        x.stage_prepare(p)
    sg, so = g.read_sim_values(), o.read_sim_values()
    assert sg.num_bodies == so.num_bodies == n
    assert np.array_equal(sim_bounds(sg), sim_bounds(so))
    assert np.array_equal(g.read_index(), o.read_index())
    assert np.array_equal(g.read_morton(), o.read_morton())

    for x in (g, o):
        x.stage_sort()
    kg = g.read_morton()
    assert np.all(kg[1:] >= kg[:-1])
    assert np.array_equal(kg, o.read_morton())
    del kg
    assert np.array_equal(g.read_index(), o.read_index())
    assert g.read_stats().error_word == 0

    for x in (g, o):
        x.stage_build()
    topo = ["child_a", "child_b", "bodies_contained", "parent_id", "node_depth", "ready_children"]
    _equal_in_chunks(lambda c, f: g.read_internal_nodes(c, f), lambda c, f: o.read_internal_nodes(c, f), n - 1,
                     topo, [], "build")

    for x in (g, o):
        x.stage_fill()
    words = ["node_depth", "ready_children", "child_a", "child_b", "parent_id", "bodies_contained"]
    _equal_in_chunks(lambda c, f: g.read_internal_nodes(c, f), lambda c, f: o.read_internal_nodes(c, f), n - 1,
                     words, ["com_mass", "aabb"], "fill internal")
    _equal_in_chunks(lambda c, f: g.read_leaf_nodes(c, f), lambda c, f: o.read_leaf_nodes(c, f), n,
                     words, ["com_mass", "aabb"], "fill leaf")
    sg, so = g.read_stats(), o.read_stats()
    assert sg.tree_height == so.tree_height
    assert sg.error_word == 0

    for x in (g, o):
        x.stage_walk(p)
    e = rel_err(g.read_accel()[:, :3], o.read_accel()[:, :3])
    assert np.median(e) < 1e-5, np.median(e)
    assert np.percentile(e, 99) < 1e-3, np.percentile(e, 99)
    sg, so = g.read_stats(), o.read_stats()
    assert abs(int(sg.interactions) - int(so.interactions)) <= 1e-4 * so.interactions
    assert sg.error_word == 0
    o.close()


def test_c4_step_graph_equals_stages(gbh_lib, c4_bodies):
    n = N_C4
    bounds = ic.exact_bounds(c4_bodies)
    p = _c4_params()
    a = BarnesHut(n, bounds, abi.units(G=1.0))
    a.upload_bodies(c4_bodies)
    a.init()
    for _ in range(2):
        a.step(p)  # the bench's path: one graph launch, in-order positions from the second step
    a.synchronize()
    ba, ia, ka = a.read_bodies().view(np.uint32), a.read_index(), a.read_morton()
    del a
    c = BarnesHut(n, bounds, abi.units(G=1.0))
    c.upload_bodies(c4_bodies)
    c.init()
    for _ in range(2):
        c.stage_reset(p)
        c.stage_prepare(p)
        c.stage_sort()
        c.stage_build()
        c.stage_fill()
        c.stage_walk(p)
        c.stage_merge(p)
        c.stage_swap()
    assert c.read_stats().error_word == 0
    assert np.array_equal(ba, c.read_bodies().view(np.uint32))
    assert np.array_equal(ia, c.read_index())
    assert np.array_equal(ka, c.read_morton())


def _c2_bodies():
    b = ic.uniform_merge(N_C2, seed=1)
    # out-of-bounds kills inside the compared steps: 500 bodies already
    # outside the box, 500 on its face moving out
    b["pos_mass"][:500, 0] = 2.5
    b["pos_mass"][500:1000, 0] = 1.9995
    b["vel_density"][500:1000, 0] = 1.0
    return b


def test_c2_merge_steps_match_oracle(gbh_lib, oracle_mod):
    n = N_C2
    bounds = np.array([-2, -2, -2, 2, 2, 2], np.float32)
    units = abi.units(G=1.0)
    p = abi.step_params(dt=5e-4, theta=0.7, softening=0.01 ** 2, mode=abi.MODE_MERGE, bounds=abi.BOUNDS_STATIC)
    g = BarnesHut(n, bounds, units)
    o = oracle_mod.OracleBarnesHut(n, bounds, units)
    b = _c2_bodies()
    for x in (g, o):
        x.upload_bodies(b)
        x.init()
    total_merged = total_oob = 0
    for step in range(6):
        # the oracle starts this step from the GPU's state
        o.upload_bodies(g.read_bodies())
        o.write_index(g.read_index())
        o.write_sim_values(g.read_sim_values())
        g.step(p)
        o.step(p)
        g.synchronize()
        tg, to = g.read_merge_tasks(), o.read_merge_tasks()
        assert set(map(tuple, tg.tolist())) == set(map(tuple, to.tolist())), step
        sg, so = g.read_stats(), o.read_stats()
        assert sg.merged == so.merged, step
        assert sg.out_of_bounds == so.out_of_bounds, step
        assert sg.error_word == 0
        assert g.read_sim_values().out_of_bounds == o.read_sim_values().out_of_bounds, step
        bg, bo = g.read_bodies(), o.read_bodies()
        assert np.array_equal(bg["pos_mass"][:, 3] == 0, bo["pos_mass"][:, 3] == 0), step
        np.testing.assert_allclose(bg["pos_mass"], bo["pos_mass"], rtol=1e-5, atol=1e-6)
        total_merged += sg.merged
        total_oob += sg.out_of_bounds
    assert total_merged >= 30 and total_oob >= 1000, (total_merged, total_oob)
    # the next compaction removes the same bodies
    for x in (g, o):
        x.stage_reset(p)
        x.stage_prepare(p)
    assert g.read_sim_values().num_bodies == o.read_sim_values().num_bodies
    o.close()
