"""The group-θ walk against a numpy restatement of it.

The group walk (k_walk_group.cu) starts each body group from its start list
(the group's own leaves and the siblings of its ancestors, k_group_paths)
rather than from the root; the accepted and listed nodes must be exactly those
of a walk from the root.  Here each group is walked from the root in numpy on
the GPU's own tree (read back after the walk): the group box, the group rule
(accept when the boxes are disjoint and half_side^2 < theta^2 (d^2 + soft),
d the distance from the centre of mass to the group's bounding sphere), every
leaf listed, the forces summed in float64.  The interaction count and the
accelerations must agree (the float32 rule can flip a node that sits on the
threshold, so both carry a small tolerance).
"""
import numpy as np
import pytest

from gravity_gb300 import BarnesHut, abi, ic

pytestmark = pytest.mark.gpu

GROUP_MAX = 96


def _groups(internal, N, n):
    """(first slot, count) of every maximal subtree of at most GROUP_MAX bodies."""
    if n <= GROUP_MAX:
        return [(0, n)]
    out = []
    stack = [N]
    while stack:
        g = stack.pop()
        nd = internal[g - N]
        for c in (int(nd["child_a"]), int(nd["child_b"])):
            if c < N:
                out.append((c, 1))
            else:
                cnt = int(internal[c - N]["bodies_contained"])
                if cnt <= GROUP_MAX:
                    k = c
                    while k >= N:
                        k = int(internal[k - N]["child_a"])
                    out.append((k, cnt))
                else:
                    stack.append(c)
    return out


def _group_walk(internal, leaves, N, first, count, theta, soft):
    """List entries (ids) of one group's walk from the root (order free)."""
    pos = leaves["com_mass"][first:first + count, :3].astype(np.float32)
    bmin, bmax = pos.min(axis=0), pos.max(axis=0)
    c = np.float32(0.5) * (bmin + bmax)
    h = np.float32(0.5) * (bmax - bmin)
    R = np.float32(np.sqrt(np.float32(h @ h)))
    listed = []
    stack = [N]
    th2 = np.float32(theta) * np.float32(theta)
    while stack:
        k = stack.pop()
        if k < N:
            listed.append(k)
            continue
        nd = internal[k - N]
        cm = nd["com_mass"][:3].astype(np.float32)
        box = nd["aabb"].astype(np.float32)
        d = cm - c
        D = np.float32(np.sqrt(np.float32(d @ d)))
        dd = max(np.float32(D - R), np.float32(0.0))
        soft_d2 = dd * dd + np.float32(soft)
        half = np.float32(0.5) * np.max(box[3:] - box[:3])
        gap = np.maximum(np.float32(0.0), np.maximum(box[:3] - bmax, bmin - box[3:]))
        if half * half < th2 * soft_d2 and float(gap @ gap) > 0.0:
            listed.append(k)
        else:
            stack.extend((int(nd["child_a"]), int(nd["child_b"])))
    return listed


@pytest.mark.parametrize("n,theta", [(50, 0.6), (97, 0.6), (1001, 0.3), (12001, 0.6)])
def test_group_theta_walk_matches_restatement(gbh_lib, n, theta):
    # 50 bodies: the whole tree is one group; 97: the root's children are
    # groups; larger trees have groups at many depths
    bodies = ic.plummer(n, seed=7)
    soft = 1e-4
    sim = BarnesHut(n, ic.exact_bounds(bodies), abi.units(G=1.0))
    sim.upload_bodies(bodies)
    sim.init()
    acc = sim.evaluate_walk(abi.step_params(theta=theta, softening=soft, mac=abi.MAC_GROUP)).astype(np.float64)
    st = sim.read_stats()
    assert st.error_word == 0 and st.frontier_saturated == 0
    N = sim.n
    live = sim.read_sim_values().num_bodies
    leaves = sim.read_leaf_nodes()
    internal = sim.read_internal_nodes()
    idx = sim.read_index()
    groups = _groups(internal, N, live)
    assert sum(c for _, c in groups) == live
    inter = 0
    ref = np.zeros((N, 3))
    for first, count in groups:
        ids = _group_walk(internal, leaves, N, first, count, theta, soft)
        inter += len(ids) * count
        src = np.array([leaves[k]["com_mass"] if k < N else internal[k - N]["com_mass"] for k in ids], np.float64)
        x = leaves["com_mass"][first:first + count, :3].astype(np.float64)
        r = src[None, :, :3] - x[:, None, :]
        w = src[None, :, 3] * (np.sum(r * r, axis=2) + soft) ** -1.5
        ref[idx[first:first + count]] = np.sum(w[:, :, None] * r, axis=1)
    assert abs(int(st.interactions) - inter) <= 1e-4 * inter, (int(st.interactions), inter)
    body = idx[:live]
    e = np.linalg.norm(acc[body] - ref[body], axis=1) / np.linalg.norm(ref[body], axis=1)
    assert np.median(e) < 1e-5, np.median(e)
    assert np.percentile(e, 99.9) < 1e-3, np.percentile(e, 99.9)


def test_group_walk_on_a_tree_built_for_the_plain_walk(gbh_lib):
    # the start lists are built with the tree when a group walk is selected;
    # a group walk on a tree built under the plain walk's parameters builds
    # them itself, and a graph-launched plain step leaves them marked stale
    n = 20000
    bodies = ic.plummer(n, seed=8)
    bounds = ic.exact_bounds(bodies)
    p_plain = abi.step_params(theta=0.5, softening=1e-4, flags=abi.FLAG_STORE_ACCEL)
    p_group = abi.step_params(theta=0.5, softening=1e-4, mac=abi.MAC_GROUP, flags=abi.FLAG_STORE_ACCEL)
    a = BarnesHut(n, bounds, abi.units(G=1.0))
    a.upload_bodies(bodies)
    a.init()
    for p in (p_group, p_plain, p_group, p_plain):  # graphs captured, then replayed
        a.step(p)
    a.synchronize()
    state = a.read_bodies()
    for x in (p_plain,):
        a.stage_reset(x)
        a.stage_prepare(x)
    a.stage_sort()
    a.stage_build()  # under the plain walk's parameters: no start lists
    a.stage_fill()
    a.stage_walk(p_group)
    st = a.read_stats()
    assert st.error_word == 0
    acc = a.read_accel()[:, :3]
    c = BarnesHut(n, bounds, abi.units(G=1.0))
    c.upload_bodies(state)
    c.init()
    ref = c.evaluate_walk(p_group)
    assert int(c.read_stats().interactions) == int(st.interactions)
    assert np.array_equal(acc, ref)
