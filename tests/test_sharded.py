"""The sharded step's host orchestration (gravity_gb300.sharded.ShardedStep)
on CPU ranks: world-size 2 and 3 gloo process groups, each rank driving the CPU
oracle's restatement of the shard entry points (rank r walks sorted slots
[n r / W, n (r + 1) / W); the updated bodies and the merge tasks are
all-gathered).  After three steps with merges and out-of-bounds kills, every
rank's state must be bit-identical to three unsharded steps on one rank."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STEPS = 3


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case():
    from gravity_gb300 import abi, ic

    n = 6000
    b = ic.uniform_merge(n, seed=9)
    b["pos_mass"][:, :3] *= 0.1  # dense: merges
    b["pos_mass"][:40, 0] = 3.0  # outside the box: killed
    b["pos_mass"][40:80, 0] = 1.9999
    b["vel_density"][40:80, 0] = 2.0  # leaving it during the steps
    bounds = np.array([-2, -2, -2, 2, 2, 2], np.float32)
    p = abi.step_params(dt=5e-4, theta=0.7, softening=1e-8, mode=abi.MODE_MERGE, bounds=abi.BOUNDS_STATIC)
    return b, bounds, p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), OMP_NUM_THREADS="2")
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from gravity_gb300 import abi
    from gravity_gb300.sharded import ShardedStep
    from oracle import oracle as O

    dist.init_process_group("gloo", rank=rank, world_size=world)
    b, bounds, p = _case()
    o = O.OracleBarnesHut(len(b), bounds, abi.units(G=1.0))
    o.upload_bodies(b)
    o.init()
    sh = ShardedStep(o)
    info = [sh.step(p) for _ in range(STEPS)]
    q.put((rank, o.read_bodies().tobytes(), o.read_index().tobytes(), o.read_sim_values().out_of_bounds,
           [i["tasks"] for i in info], [i["ranges"] for i in info]))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_steps_equal_one_rank(oracle_mod, world):
    torch = pytest.importorskip("torch")
    from gravity_gb300 import abi

    b, bounds, p = _case()
    ref = oracle_mod.OracleBarnesHut(len(b), bounds, abi.units(G=1.0))
    ref.upload_bodies(b)
    ref.init()
    merged = 0
    for _ in range(STEPS):
        ref.step(p)
        merged += ref.read_stats().merged
    assert merged > 10 and ref.read_sim_values().out_of_bounds >= 40
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for x in ps:
        x.start()
    got = [q.get(timeout=300) for _ in range(world)]
    for x in ps:
        x.join(timeout=60)
        assert x.exitcode == 0
    want_b = ref.read_bodies().tobytes()
    want_i = ref.read_index().tobytes()
    for rank, bodies, index, oob, tasks, ranges in got:
        assert bodies == want_b, rank
        assert index == want_i, rank
        assert oob == ref.read_sim_values().out_of_bounds, rank
        assert sum(tasks) > 0
        for rr in ranges:  # the shares tile the live slots in rank order
            assert rr[0][0] == 0 and all(rr[k][1] == rr[k + 1][0] for k in range(world - 1))
