"""Known-answer tests of the CPU oracle from the mathematics of the method
(the reference ships no tests).  They pin the oracle independently of the
reference harness: Morton interleave and quantisation, the Karras longest
common prefix with its index tie-break, two- and three-body accelerations,
conservation in a merge, and the Plummer enclosed-mass field."""
import numpy as np
import pytest

from gravity_gb300 import abi, ic


def test_expand_and_interleave(oracle_mod):
    O = oracle_mod
    assert O.morton3d64(0, 0, 0) == 0
    # x occupies bit 3k+2, y bit 3k+1, z bit 3k (bh_morton.comp:18-21)
    assert O.morton3d64(1, 0, 0) == 0b100
    assert O.morton3d64(0, 1, 0) == 0b010
    assert O.morton3d64(0, 0, 1) == 0b001
    full = (1 << 21) - 1
    assert O.morton3d64(full, full, full) == (1 << 63) - 1
    assert O.morton3d64(full, 0, 0) == 0x4924924924924924
    # random cross-check against a bit-by-bit interleave
    rng = np.random.default_rng(0)
    for _ in range(200):
        x, y, z = (int(v) for v in rng.integers(0, 1 << 21, 3))
        want = 0
        for k in range(21):
            want |= ((x >> k) & 1) << (3 * k + 2) | ((y >> k) & 1) << (3 * k + 1) | ((z >> k) & 1) << (3 * k)
        assert O.morton3d64(x, y, z) == want


def test_morton_encode_box_points(oracle_mod):
    O = oracle_mod
    mn, mx = [-1.0, -1.0, -1.0], [1.0, 1.0, 1.0]
    full = (1 << 21) - 1
    assert O.morton_encode([-1, -1, -1], mn, mx) == 0
    assert O.morton_encode([1, 1, 1], mn, mx) == O.morton3d64(full, full, full)
    half = int(np.floor(np.float32(0.5) * np.float32(2097151.0)))
    assert O.morton_encode([0, 0, 0], mn, mx) == O.morton3d64(half, half, half)
    # outside the box clamps to the faces; NaN maps to the box centre
    assert O.morton_encode([5, -5, 0], mn, mx) == O.morton3d64(full, 0, half)
    assert O.morton_encode([np.nan, 0, 0], mn, mx) == O.morton3d64(half, half, half)
    assert O.morton_encode([np.inf, 0, 0], mn, mx) == O.morton3d64(half, half, half)
    # an empty box (min > max) maps everything to its centre (bh_morton.comp:253-254)
    c = O.morton_encode([0.3, 0.1, 0.2], [1, 1, 1], [-1, -1, -1])
    assert c == O.morton_encode([0, 0, 0], [1, 1, 1], [-1, -1, -1])


def test_lcp_with_index_tiebreak(oracle_mod):
    O = oracle_mod
    keys = np.array([0b0001, 0b0001, 0b0011, 0b1000], dtype=np.uint64)
    assert O.safe_lcp(keys, 0, 4) == -1 and O.safe_lcp(keys, -1, 0) == -1
    # distinct keys: clz64(a ^ b)
    assert O.safe_lcp(keys, 1, 2) == 64 - 2
    assert O.safe_lcp(keys, 2, 3) == 64 - 4
    # equal keys: 64 + clz32(i ^ j)  (bh_tree.comp:27-35)
    assert O.safe_lcp(keys, 0, 1) == 64 + 31
    assert O.safe_lcp(keys, 0, 0) == 64


def _tree_for_keys(O, keys):
    """Build the tree of given sorted keys through the oracle stage API."""
    n = len(keys)
    bodies = np.zeros(n, dtype=abi.BODY_DTYPE)
    bodies["pos_mass"][:, 3] = 1.0
    bodies["vel_density"][:, 3] = 1.0
    o = O.OracleBarnesHut(n, [-1, -1, -1, 1, 1, 1], abi.units(G=1.0))
    o.upload_bodies(bodies)
    o.init()
    s = o.read_sim_values()
    s.num_bodies = n
    o.write_sim_values(s)
    o.write_morton(np.asarray(keys, np.uint64))
    o.stage_build()
    return o.read_internal_nodes()[: n - 1], o.read_leaf_nodes()


def _check_binary_tree(internal, leaf, n):
    N = n
    seen_leaf = np.zeros(n, int)
    seen_int = np.zeros(max(n - 1, 1), int)
    for i, nd in enumerate(internal):
        for c in (nd["child_a"], nd["child_b"]):
            if c < N:
                seen_leaf[c] += 1
                assert leaf[c]["parent_id"] == i + N
            else:
                seen_int[c - N] += 1
                assert internal[c - N]["parent_id"] == i + N
        lo_hi = []
        # the range of node i covers bodies_contained consecutive leaves
    assert np.all(seen_leaf == 1)
    assert seen_int[0] == 0 and np.all(seen_int[1:] == 1)
    assert internal[0]["parent_id"] == 0xFFFFFFFF
    assert internal[0]["bodies_contained"] == n


@pytest.mark.parametrize("keys", [[0, 1], [0, 1, 2], [1, 2, 4, 5, 19, 24, 25, 30], [7, 7, 7, 7, 7], [0, 0, 3, 3, 3, 9]])
def test_karras_small_trees(oracle_mod, keys):
    internal, leaf = _tree_for_keys(oracle_mod, keys)
    _check_binary_tree(internal, leaf, len(keys))


def test_karras_paper_example(oracle_mod):
    # Karras 2012, figure 3: keys 00001 00010 00100 00101 10011 11000 11001 11110
    keys = [0b00001, 0b00010, 0b00100, 0b00101, 0b10011, 0b11000, 0b11001, 0b11110]
    internal, leaf = _tree_for_keys(oracle_mod, keys)
    N = 8
    kids = [(int(a), int(b)) for a, b in zip(internal["child_a"], internal["child_b"])]
    # root splits between 3 and 4: children internal 3 and internal 4
    assert kids[0] == (3 + N, 4 + N)
    assert kids[3] == (1 + N, 2 + N)
    assert kids[4] == (4, 5 + N)
    assert kids[1] == (0, 1)
    assert kids[2] == (2, 3)
    assert kids[5] == (6 + N, 7)
    assert kids[6] == (5, 6)


def _walk_accel(O, bodies, theta=0.5, soft=0.0, G=1.0):
    n = len(bodies)
    p = ic.exact_bounds(bodies)
    o = O.OracleBarnesHut(n, p, abi.units(G=G))
    o.upload_bodies(bodies)
    o.init()
    o.step(abi.step_params(dt=0.0, theta=theta, softening=soft, flags=abi.FLAG_STORE_ACCEL))
    return o.read_accel()[:, :3], o


def test_two_body_acceleration(oracle_mod):
    b = ic.pack(np.array([[0.0, 0, 0], [2.0, 0, 0]]), np.zeros((2, 3)), np.array([3.0, 5.0]), np.ones(2))
    a, _ = _walk_accel(oracle_mod, b, soft=0.0)
    np.testing.assert_allclose(a[0], [5.0 / 4.0, 0, 0], rtol=1e-6)
    np.testing.assert_allclose(a[1], [-3.0 / 4.0, 0, 0], rtol=1e-6)


def test_three_body_leaves_exact(oracle_mod):
    pos = np.array([[0.0, 0, 0], [1.0, 0, 0], [0.0, 2.0, 0]])
    m = np.array([1.0, 2.0, 4.0])
    b = ic.pack(pos, np.zeros((3, 3)), m, np.ones(3))
    soft = 1e-3
    a, _ = _walk_accel(oracle_mod, b, theta=1e-6, soft=soft)  # theta -> 0: every leaf is visited
    for i in range(3):
        want = np.zeros(3)
        for j in range(3):
            if i != j:
                r = pos[j] - pos[i]
                want += m[j] * r / (r @ r + soft) ** 1.5
        np.testing.assert_allclose(a[i], want, rtol=1e-5)


def test_plummer_enclosed_mass_field(oracle_mod):
    # the tree acceleration of a Plummer sphere follows -G M r / (r^2 + a^2)^1.5
    n = 30000
    b = ic.plummer(n, seed=8)
    a, _ = _walk_accel(oracle_mod, b, theta=0.3, soft=1e-4)
    pos = b["pos_mass"][:, :3].astype(np.float64)
    r = np.linalg.norm(pos, axis=1)
    sel = (r > 0.3) & (r < 2.0)
    want = -pos[sel] / ((r[sel] ** 2 + 1.0) ** 1.5)[:, None]
    got = a[sel]
    radial = np.sum(got * pos[sel], axis=1) / r[sel]
    radial_want = np.sum(want * pos[sel], axis=1) / r[sel]
    # Poisson noise of a 30k-body realisation: compare the median ratio
    assert abs(np.median(radial / radial_want) - 1.0) < 0.03


def test_merge_conserves_mass_momentum_volume(oracle_mod):
    pos = np.array([[0.0, 0, 0], [0.0015, 0, 0]])
    vel = np.array([[1.0, 0, 0], [-1.0, 0.5, 0]])
    m = np.array([1e-3, 5e-4])
    rho = np.array([ic.MERGE_DENSITY, ic.MERGE_DENSITY / 2])
    b = ic.pack(pos, vel, m, rho)
    o = oracle_mod.OracleBarnesHut(2, [-1, -1, -1, 1, 1, 1], abi.units(G=1.0))
    o.upload_bodies(b)
    o.init()
    o.step(abi.step_params(dt=0.0, theta=0.5, softening=1e-12, mode=abi.MODE_MERGE, bounds=abi.BOUNDS_STATIC))
    out = o.read_bodies()
    live = out["pos_mass"][:, 3] != 0
    assert live.sum() == 1
    w = out[live][0]
    M = m.sum()
    np.testing.assert_allclose(w["pos_mass"][3], M, rtol=1e-6)
    np.testing.assert_allclose(w["pos_mass"][:3], (pos * m[:, None]).sum(0) / M, rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(w["vel_density"][:3], (vel * m[:, None]).sum(0) / M, rtol=1e-5)
    np.testing.assert_allclose(w["vel_density"][3], M / (m / rho).sum(), rtol=1e-5)


def test_dead_partition_is_stable(oracle_mod):
    n = 1000
    b = ic.plummer(n, seed=1)
    dead = np.arange(0, n, 7)
    b["pos_mass"][dead, 3] = 0
    o = oracle_mod.OracleBarnesHut(n, ic.exact_bounds(b), abi.units(G=1.0))
    o.upload_bodies(b)
    o.init()
    p = abi.step_params()
    o.stage_reset(p)
    o.stage_partition()
    idx = o.read_index()
    alive = np.setdiff1d(np.arange(n), dead)
    assert np.array_equal(idx[: len(alive)], alive)
    assert np.array_equal(idx[len(alive):], dead)
    assert o.read_sim_values().just_died == len(dead)
    assert np.all(o.read_bodies(abi.BODIES_IN)[dead].view(np.uint32) == 0)
    assert np.all(o.read_bodies(abi.BODIES_OUT)[dead].view(np.uint32) == 0)


def test_direct_sum_fp64_two_bodies(oracle_mod):
    b = ic.pack(np.array([[0.0, 0, 0], [0, 3.0, 0]]), np.zeros((2, 3)), np.array([2.0, 1.0]), np.ones(2))
    a = oracle_mod.direct_sum_fp64(b, np.array([0, 1], np.uint32), 1.0, 0.0)
    np.testing.assert_allclose(a, [[0, 1.0 / 9, 0], [0, -2.0 / 9, 0]], rtol=1e-12)
