"""The sharded step: one BarnesHut.step split over the ranks of a
torch.distributed process group, one process per GPU.

Every rank holds the whole state and builds the same tree; each walks its
share of the live bodies (gbh_step_shard_walk); the ranks then all-gather the
updated bodies (in sorted-slot order) and the merge tasks, every rank installs
the others' bodies, writes the union of the tasks and finishes the step
(merge resolution and swap).  The reference walks each body independently of
the others (src/main/resources/shaders/compute/force/bh_force.comp:40-142), so
the state after the step is bit for bit that of one unsharded step, on every
rank.

The exchange per step is the walk's output: 36 bytes per live body (position,
mass, velocity, density and the magnitude of the body's acceleration, which
the learned criterion reads in the next step; velocities travel too, because
the shares move as the bodies' sorted order changes) plus the merge tasks.  The simulation object is
anything with the step_shard_* methods: gravity_gb300.BarnesHut (the GPU, with
NCCL or gloo device all-gathers) or a CPU restatement with the same methods.
"""
from __future__ import annotations

import numpy as np

from . import abi


class ShardedStep:
    def __init__(self, sim, group=None):
        import torch.distributed as dist

        self.sim = sim
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)

    def step(self, params: abi.StepParams) -> dict:
        import torch

        dist, g = self.dist, self.group
        lo, hi = self.sim.step_shard_walk(params, self.rank, self.world)
        ranges = [None] * self.world
        dist.all_gather_object(ranges, (lo, hi), group=g)
        # the updated bodies, padded to the largest share
        per = self.sim.shard_bytes_per_body
        width = max(h - l for l, h in ranges) * per
        mine = self.sim.shard_pack_tensor(lo, hi)
        send = torch.zeros(max(width, 1), dtype=torch.uint8, device=mine.device)
        send[: mine.numel()] = mine
        parts = [torch.empty_like(send) for _ in range(self.world)]
        dist.all_gather(parts, send, group=g)
        for r, (l, h) in enumerate(ranges):
            if r != self.rank and h > l:
                self.sim.shard_unpack_tensor(l, parts[r][: (h - l) * per])
        # the merge tasks of every rank, in ordering-key order
        tasks = [None] * self.world
        dist.all_gather_object(tasks, self.sim.read_merge_tasks_full(), group=g)
        pairs = np.concatenate([t[0] for t in tasks]).reshape(-1, 2)
        keys = np.concatenate([t[1] for t in tasks])
        slots = np.concatenate([t[2] for t in tasks])
        order = np.argsort(keys, kind="stable")
        self.sim.write_merge_tasks(pairs[order], keys[order], slots[order])
        # out-of-bounds kills of the other ranks
        oob = int(self.sim.read_stats().out_of_bounds)
        counts = [None] * self.world
        dist.all_gather_object(counts, oob, group=g)
        self.sim.step_shard_finish(sum(counts) - oob)
        return {"range": (lo, hi), "ranges": ranges, "tasks": int(len(keys)), "out_of_bounds": sum(counts)}
