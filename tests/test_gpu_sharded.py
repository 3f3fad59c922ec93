"""The sharded step's entry points on the GPU (gbh_step_shard_walk,
gbh_shard_pack/unpack, gbh_read/write_merge_tasks, gbh_step_shard_finish).
Two or three contexts on one GPU stand in for the ranks; the host runs them
one after another and exchanges their packed bodies and merge tasks, as an
all-gather would (no kernel waits on another context).  After three steps the
state of every context must equal, bit for bit, three unsharded graph steps,
for the plain walk with merges and out-of-bounds kills, the group walk and the
learned walk."""
import numpy as np
import pytest

from gravity_gb300 import BarnesHut, abi, ic

pytestmark = pytest.mark.gpu

STEPS = 3


def _case(n=120000):
    b = ic.uniform_merge(n, seed=9)
    b["pos_mass"][:, :3] *= 0.1
    b["pos_mass"][:200, 0] = 3.0
    b["pos_mass"][200:400, 0] = 1.9999
    b["vel_density"][200:400, 0] = 2.0
    return b, np.array([-2, -2, -2, 2, 2, 2], np.float32)


def _sharded_step(sims, p):
    world = len(sims)
    per = abi.SHARD_BYTES_PER_BODY
    ranges = [s.step_shard_walk(p, r, world) for r, s in enumerate(sims)]
    packed = [s.shard_pack_tensor(lo, hi) for s, (lo, hi) in zip(sims, ranges)]
    for r, s in enumerate(sims):
        for q, (lo, hi) in enumerate(ranges):
            if q != r and hi > lo:
                assert packed[q].numel() == (hi - lo) * per
                s.shard_unpack_tensor(lo, packed[q])
    tasks = [s.read_merge_tasks_full() for s in sims]
    pairs = np.concatenate([t[0] for t in tasks]).reshape(-1, 2)
    keys = np.concatenate([t[1] for t in tasks])
    slots = np.concatenate([t[2] for t in tasks])
    oob = [int(s.read_stats().out_of_bounds) for s in sims]
    for r, s in enumerate(sims):
        s.write_merge_tasks(pairs, keys, slots)
        s.step_shard_finish(sum(oob) - oob[r])
    assert ranges[0][0] == 0 and all(ranges[k][1] == ranges[k + 1][0] for k in range(world - 1))
    return len(keys)


def _weights(b, bounds, p):
    w = BarnesHut(len(b), bounds, abi.units(G=1.0))
    w.upload_bodies(b)
    w.init()
    q = abi.StepParams.from_buffer_copy(p)
    q.merging_collision_or_neither = abi.MODE_NEITHER
    w.mac_generate(q, max_pairs=50000, seed=1)
    w.mac_train(epochs=2, batch=4096, lr=3e-3, seed=0)
    return w.mac_get_weights()


@pytest.mark.parametrize("mac,world", [(abi.MAC_PLAIN, 2), (abi.MAC_PLAIN, 3), (abi.MAC_GROUP, 2),
                                       (abi.MAC_LEARNED, 2)])
def test_sharded_steps_equal_unsharded(gbh_lib, mac, world):
    torch = pytest.importorskip("torch")
    b, bounds = _case()
    p = abi.step_params(dt=5e-4, theta=0.7 if mac == abi.MAC_PLAIN else 0.5, softening=1e-8, mode=abi.MODE_MERGE,
                        bounds=abi.BOUNDS_STATIC, mac=mac, mac_tolerance=-2.5)
    weights = _weights(b, bounds, p) if mac == abi.MAC_LEARNED else None
    sims = []
    for _ in range(world + 1):
        s = BarnesHut(len(b), bounds, abi.units(G=1.0))
        s.upload_bodies(b)
        s.init()
        if weights is not None:
            s.mac_set_weights(weights)
        sims.append(s)
    ref, ranks = sims[0], sims[1:]
    tasks = 0
    for _ in range(STEPS):
        ref.step(p)
        tasks += _sharded_step(ranks, p)
    ref.synchronize()
    assert tasks > 0
    want = ref.read_bodies().view(np.uint32)
    for r, s in enumerate(ranks):
        assert s.read_stats().error_word == 0
        assert np.array_equal(s.read_bodies().view(np.uint32), want), r
        assert np.array_equal(s.read_index(), ref.read_index()), r
        assert s.read_sim_values().out_of_bounds == ref.read_sim_values().out_of_bounds >= 200, r
    # a graph step after the sharded ones continues from the same state
    ref.step(p)
    ranks[0].step(p)
    ref.synchronize()
    assert np.array_equal(ranks[0].read_bodies().view(np.uint32), ref.read_bodies().view(np.uint32))
