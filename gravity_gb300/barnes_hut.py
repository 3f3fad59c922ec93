"""Host-side mirror of the reference's BarnesHut step interface over libgbh.so.

The reference drives its GLSL pipeline from Java
(src/main/java/com/grumbo/simulation/BarnesHut.java:99-173, GPU.java:172-1196).
`BarnesHut` keeps that interface: construct with the body capacity, bounds and
unit set (GPU.initGPU), upload bodies (GPU.uploadPlanetsData), `init()` and
`step()`.  The per-stage methods carry the reference's stage names and run the
stage entry points of the C ABI; the compaction, bounds update and Morton
encode are one fused stage here (`partition_dead_bodies`).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from ._lib import GbhError, check, lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class BarnesHut:
    """One simulation context on one GPU (owns all its device memory)."""

    def __init__(self, initial_num_bodies: int, bounds, units: abi.Units | None = None, device: int = 0):
        self.n = int(initial_num_bodies)
        self.device = int(device)
        b = np.ascontiguousarray(np.asarray(bounds, dtype=np.float32).reshape(-1))
        if b.size != 6:
            raise ValueError("bounds must hold 6 floats (min xyz, max xyz)")
        self._bounds = (C.c_float * 6)(*b.tolist())
        self.units = units if units is not None else abi.units()
        h = C.c_void_p()
        rc = lib().gbh_create(C.byref(h), self.n, self._bounds, C.byref(self.units), device)
        if rc != 0:
            raise GbhError(rc, (lib().gbh_last_error(None) or b"").decode())
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            lib().gbh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _chk(self, rc):
        check(rc, self._h)

    # ---- lifecycle (GPU.initGPU / BarnesHut.init / BarnesHut.step) ----------
    def upload_bodies(self, bodies: np.ndarray, offset: int = 0, chunk: int = 1 << 22):
        b = np.ascontiguousarray(bodies, dtype=abi.BODY_DTYPE)
        for s in range(0, len(b), chunk):
            part = b[s : s + chunk]
            self._chk(lib().gbh_upload_bodies(self._h, _ptr(part), len(part), offset + s))

    def exchange_bodies(self, out: np.ndarray, bodies: np.ndarray, offset: int = 0):
        """Read the current bodies into `out` and install `bodies` in their
        place, the two copies overlapped (gbh_exchange_bodies)."""
        b = np.ascontiguousarray(bodies, dtype=abi.BODY_DTYPE)
        if out.dtype != abi.BODY_DTYPE or len(out) < len(b) or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous BODY_DTYPE array of at least len(bodies) bodies")
        self._chk(lib().gbh_exchange_bodies(self._h, _ptr(out), _ptr(b), len(b), offset))
        return out

    def _whole_state(self, a: np.ndarray | None, what: str, writable: bool):
        if a is None:
            return None
        if a.dtype != abi.BODY_DTYPE or len(a) != self.n or not a.flags.c_contiguous or (writable and not a.flags.writeable):
            raise ValueError(f"{what} must be a contiguous BODY_DTYPE array of initial_num_bodies bodies")
        return a

    def step_streamed(self, params: abi.StepParams, next_input: np.ndarray | None, last_result: np.ndarray | None):
        """One step on the current state; while it runs, `next_input` goes to
        the device (it becomes the state after this step) and the previous
        call's result comes back into `last_result` (gbh_step_streamed)."""
        nxt = self._whole_state(next_input, "next_input", False)
        out = self._whole_state(last_result, "last_result", True)
        self._chk(lib().gbh_step_streamed(self._h, C.byref(params), None if nxt is None else _ptr(nxt),
                                          None if out is None else _ptr(out)))
        return last_result

    def step_streamed_finish(self, last_result: np.ndarray | None):
        """The last streamed step's result (gbh_step_streamed_finish)."""
        out = self._whole_state(last_result, "last_result", True)
        self._chk(lib().gbh_step_streamed_finish(self._h, None if out is None else _ptr(out)))
        return last_result

    # ---- the sharded step (gbh_step_shard_*; orchestrated by sharded.ShardedStep)
    def step_shard_walk(self, params: abi.StepParams, rank: int, world: int) -> tuple[int, int]:
        """Tree of the whole state and this rank's share of the walk; returns
        the sorted slots [lo, hi) it updated."""
        r = (C.c_uint32 * 2)()
        self._chk(lib().gbh_step_shard_walk(self._h, C.byref(params), rank, world, r))
        return int(r[0]), int(r[1])

    shard_bytes_per_body = abi.SHARD_BYTES_PER_BODY

    def shard_pack_tensor(self, lo: int, hi: int):
        """The updated bodies of slots [lo, hi), slot order, and their |a|, as
        a uint8 tensor on this context's GPU (the all-gather's send buffer)."""
        import torch

        t = torch.empty((hi - lo) * abi.SHARD_BYTES_PER_BODY, dtype=torch.uint8, device=f"cuda:{self.device}")
        self._chk(lib().gbh_shard_pack(self._h, lo, hi - lo, C.c_void_p(t.data_ptr())))
        return t

    def shard_unpack_tensor(self, lo: int, t):
        """Install another rank's bodies of slots [lo, lo + len): a uint8 tensor
        on this context's GPU, complete on torch's current stream."""
        import torch

        torch.cuda.current_stream(self.device).synchronize()
        count = t.numel() // abi.SHARD_BYTES_PER_BODY
        self._chk(lib().gbh_shard_unpack(self._h, lo, count, C.c_void_p(t.data_ptr())))

    def read_merge_tasks_full(self):
        cnt = C.c_uint32(0)
        self._chk(lib().gbh_read_merge_tasks_full(self._h, None, None, None, 0, C.byref(cnt)))
        pairs = np.zeros((cnt.value, 2), np.uint32)
        keys = np.zeros(cnt.value, np.uint64)
        slots = np.zeros(cnt.value, np.uint32)
        if cnt.value:
            self._chk(lib().gbh_read_merge_tasks_full(self._h, _ptr(pairs), _ptr(keys), _ptr(slots), cnt.value,
                                                      C.byref(cnt)))
        return pairs, keys, slots

    def write_merge_tasks(self, pairs, keys, slots):
        p = np.ascontiguousarray(pairs, np.uint32)
        k = np.ascontiguousarray(keys, np.uint64)
        s = np.ascontiguousarray(slots, np.uint32)
        self._chk(lib().gbh_write_merge_tasks(self._h, _ptr(p), _ptr(k), _ptr(s), len(k)))

    def step_shard_finish(self, out_of_bounds_other_ranks: int):
        self._chk(lib().gbh_step_shard_finish(self._h, int(out_of_bounds_other_ranks)))

    def generate_bodies(self, params: abi.IcParams, seed: int = 0, count: int | None = None, offset: int = 0):
        """Seeded initial conditions written on the device (gbh_generate_bodies)."""
        count = self.n - offset if count is None else count
        self._chk(lib().gbh_generate_bodies(self._h, C.byref(params), seed, count, offset))

    def init(self):
        self._chk(lib().gbh_init(self._h))

    def step(self, params: abi.StepParams, count: int = 1):
        self._chk(lib().gbh_step_n(self._h, C.byref(params), count))

    def synchronize(self):
        self._chk(lib().gbh_synchronize(self._h))

    def clear_error(self):
        self._chk(lib().gbh_clear_error(self._h))

    @property
    def stream(self) -> int:
        return lib().gbh_stream(self._h) or 0

    # ---- stages, named after BarnesHut.java's private methods ----------------
    def reset_values(self, p):
        self._chk(lib().gbh_stage_reset(self._h, C.byref(p)))

    def partition_dead_bodies(self, p):
        """partitionDeadBodies + decrementDeadBodies + updateBounds + generateMortonCodes."""
        self._chk(lib().gbh_stage_prepare(self._h, C.byref(p)))

    def radix_sort(self):
        self._chk(lib().gbh_stage_sort(self._h))

    def build_binary_radix_tree(self):
        self._chk(lib().gbh_stage_build(self._h))

    def compute_com_and_location(self):
        self._chk(lib().gbh_stage_fill(self._h))

    def compute_force(self, p):
        self._chk(lib().gbh_stage_walk(self._h, C.byref(p)))

    def merge_bodies(self, p):
        self._chk(lib().gbh_stage_merge(self._h, C.byref(p)))

    def swap_body_buffers(self):
        self._chk(lib().gbh_stage_swap(self._h))

    # short names following the C ABI's gbh_stage_* entry points
    stage_reset = reset_values
    stage_prepare = partition_dead_bodies
    stage_sort = radix_sort
    stage_build = build_binary_radix_tree
    stage_fill = compute_com_and_location
    stage_walk = compute_force
    stage_merge = merge_bodies
    stage_swap = swap_body_buffers

    def step_profiled(self, p) -> dict:
        ms = (C.c_float * abi.NUM_STAGES)()
        self._chk(lib().gbh_step_profiled(self._h, C.byref(p), ms))
        return dict(zip(abi.STAGE_NAMES, [float(x) for x in ms]))

    # ---- read-back -----------------------------------------------------------
    def read_bodies(self, which=abi.BODIES_IN, count=None, offset=0, out: np.ndarray | None = None) -> np.ndarray:
        """Bodies [offset, offset + count) of the input (or output) buffer,
        into `out` when given (a contiguous BODY_DTYPE array, e.g. pinned)."""
        count = self.n - offset if count is None else count
        if out is None:
            out = np.zeros(count, dtype=abi.BODY_DTYPE)
        elif out.dtype != abi.BODY_DTYPE or len(out) < count or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous BODY_DTYPE array of at least count bodies")
        self._chk(lib().gbh_read_bodies(self._h, which, _ptr(out), count, offset))
        return out

    def read_leaf_nodes(self, count=None, offset=0) -> np.ndarray:
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=abi.NODE_DTYPE)
        self._chk(lib().gbh_read_leaf_nodes(self._h, _ptr(out), count, offset))
        return out

    def read_internal_nodes(self, count=None, offset=0) -> np.ndarray:
        cap = max(self.n - 1, 1)
        count = cap - offset if count is None else count
        out = np.zeros(count, dtype=abi.NODE_DTYPE)
        self._chk(lib().gbh_read_internal_nodes(self._h, _ptr(out), count, offset))
        return out

    def read_sim_values(self) -> abi.SimValues:
        s = abi.SimValues()
        self._chk(lib().gbh_read_sim_values(self._h, C.byref(s)))
        return s

    def read_index(self, count=None, offset=0) -> np.ndarray:
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=np.uint32)
        self._chk(lib().gbh_read_index(self._h, _ptr(out), count, offset))
        return out

    def read_morton(self, count=None, offset=0) -> np.ndarray:
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=np.uint64)
        self._chk(lib().gbh_read_morton(self._h, _ptr(out), count, offset))
        return out

    def read_merge_tasks(self) -> np.ndarray:
        cnt = C.c_uint32(0)
        self._chk(lib().gbh_read_merge_tasks(self._h, None, 0, C.byref(cnt)))
        out = np.zeros((cnt.value, 2), dtype=np.uint32)
        if cnt.value:
            self._chk(lib().gbh_read_merge_tasks(self._h, _ptr(out), cnt.value, C.byref(cnt)))
        return out

    def read_accel(self, count=None, offset=0) -> np.ndarray:
        count = self.n - offset if count is None else count
        out = np.zeros((count, 4), dtype=np.float32)
        self._chk(lib().gbh_read_accel(self._h, _ptr(out), count, offset))
        return out

    def read_stats(self) -> abi.Stats:
        s = abi.Stats()
        self._chk(lib().gbh_read_stats(self._h, C.byref(s)))
        return s

    def device_ptrs(self) -> abi.DeviceBuffers:
        d = abi.DeviceBuffers()
        self._chk(lib().gbh_device_ptrs(self._h, C.byref(d)))
        return d

    def write_sim_values(self, s: abi.SimValues):
        self._chk(lib().gbh_write_sim_values(self._h, C.byref(s)))

    def write_index(self, idx: np.ndarray, offset=0):
        a = np.ascontiguousarray(idx, dtype=np.uint32)
        self._chk(lib().gbh_write_index(self._h, _ptr(a), len(a), offset))

    def write_morton(self, keys: np.ndarray, offset=0):
        a = np.ascontiguousarray(keys, dtype=np.uint64)
        self._chk(lib().gbh_write_morton(self._h, _ptr(a), len(a), offset))

    # ---- accuracy reference --------------------------------------------------------
    def direct_sum(self, params: abi.StepParams, sample: np.ndarray) -> np.ndarray:
        s = np.ascontiguousarray(sample, dtype=np.uint32)
        out = np.zeros((len(s), 3), dtype=np.float64)
        self._chk(lib().gbh_direct_sum(self._h, C.byref(params), _ptr(s), len(s), _ptr(out)))
        return out

    def read_potential(self, count=None, offset=0) -> np.ndarray:
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=np.float32)
        self._chk(lib().gbh_read_potential(self._h, _ptr(out), count, offset))
        return out

    def read_positions_fp64(self, count=None, offset=0) -> np.ndarray:
        """FP64 positions of the precision form, float64[count, 3] by body id."""
        count = self.n - offset if count is None else count
        out = np.zeros((count, 4), dtype=np.float64)
        self._chk(lib().gbh_read_positions_fp64(self._h, _ptr(out), count, offset))
        return out[:, :3]

    def write_positions_fp64(self, xyz: np.ndarray, offset: int = 0):
        """Set FP64 positions (float64[count, 3]) of bodies [offset, offset + count);
        their FP32 body positions become the rounded values."""
        a = np.zeros((len(xyz), 4), dtype=np.float64)
        a[:, :3] = xyz
        self._chk(lib().gbh_write_positions_fp64(self._h, _ptr(a), len(a), offset))

    def diagnostics(self, params: abi.StepParams | None = None) -> dict:
        """Mass, momentum, centre of mass, kinetic/potential/total energy and
        angular momentum of the current state in FP64.  With `params`, a walk
        of the current state (state not advanced) supplies the potential."""
        if params is not None:
            p = abi.StepParams.from_buffer_copy(params)
            p.flags |= abi.FLAG_STORE_POTENTIAL
            self.reset_values(p)
            self.partition_dead_bodies(p)
            self.radix_sort()
            self.build_binary_radix_tree()
            self.compute_com_and_location()
            self.compute_force(p)
        d = abi.Diagnostics()
        self._chk(lib().gbh_read_diagnostics(self._h, C.byref(d)))
        return abi.diagnostics_to_dict(d)

    def evaluate_walk(self, params: abi.StepParams) -> np.ndarray:
        """Accelerations of the current state under `params` (tree + walk
        stages, no merge, no swap: the state does not advance).  float[N, 3]
        by body id; stats of the walk in read_stats()."""
        p = abi.StepParams.from_buffer_copy(params)
        p.flags |= abi.FLAG_STORE_ACCEL
        self.reset_values(p)
        self.partition_dead_bodies(p)
        self.radix_sort()
        self.build_binary_radix_tree()
        self.compute_com_and_location()
        self.compute_force(p)
        return self.read_accel()[:, :3]

    # ---- learned multipole-acceptance criterion ---------------------------------
    def mac_set_weights(self, w: np.ndarray):
        a = np.ascontiguousarray(w, dtype=np.float32).reshape(-1)
        self._chk(lib().gbh_mac_set_weights(self._h, _ptr(a), len(a)))

    def mac_get_weights(self) -> np.ndarray:
        out = np.zeros(abi.MAC_NUM_PARAMS, dtype=np.float32)
        self._chk(lib().gbh_mac_get_weights(self._h, _ptr(out), len(out)))
        return out

    def mac_set_band(self, theta_accept: float, theta_open: float):
        """Group-rule thetas bounding the band the network decides."""
        self._chk(lib().gbh_mac_set_band(self._h, theta_accept, theta_open))

    def mac_get_band(self) -> tuple[float, float]:
        lo, hi = C.c_float(0), C.c_float(0)
        self._chk(lib().gbh_mac_get_band(self._h, C.byref(lo), C.byref(hi)))
        return float(lo.value), float(hi.value)

    # ---- headless node selection (the render shaders' level-of-detail pass) --
    def _select(self, fn, view: abi.View, dtype: np.dtype, capacity: int | None):
        """Runs a gbh_select_* entry point into a device buffer (a torch
        tensor) and copies the records back, sorted by node."""
        import torch

        cap = max(self.n, 1) if capacity is None else capacity
        buf = torch.empty((max(cap, 1), dtype.itemsize), dtype=torch.uint8, device=f"cuda:{self.device}")
        cnt = C.c_uint32(0)
        self._chk(fn(self._h, C.byref(view), C.c_void_p(buf.data_ptr()), cap, C.byref(cnt)))
        got = min(cnt.value, cap)
        out = buf[:got].cpu().numpy().reshape(-1).view(dtype).copy()
        return np.sort(out, order="node"), cnt.value

    def select_glow_nodes(self, view: abi.View, capacity: int | None = None):
        """(records, selected): nodeglow.vert's per-node outputs of the drawn nodes."""
        return self._select(lib().gbh_select_glow_nodes, view, abi.GLOW_SPLAT_DTYPE, capacity)

    def select_regions(self, view: abi.View, capacity: int | None = None):
        """(records, selected): regions.vert's boxes of the nodes in the depth range."""
        return self._select(lib().gbh_select_regions, view, abi.REGION_DTYPE, capacity)

    def mac_generate(self, params: abi.StepParams, max_pairs: int, seed: int = 0) -> int:
        cnt = C.c_uint32(0)
        self._chk(lib().gbh_mac_generate(self._h, C.byref(params), max_pairs, seed, C.byref(cnt)))
        return int(cnt.value)

    def mac_read_pairs(self, count: int, offset: int = 0):
        f = np.zeros((count, abi.MAC_FEATURES), dtype=np.float32)
        y = np.zeros(count, dtype=np.float32)
        self._chk(lib().gbh_mac_read_pairs(self._h, _ptr(f), _ptr(y), count, offset))
        return f, y

    def mac_read_pair_ids(self, count: int, offset: int = 0) -> np.ndarray:
        """(first sorted slot of the group, group size, node id) per pair."""
        out = np.zeros((count, 3), dtype=np.uint32)
        self._chk(lib().gbh_mac_read_pair_ids(self._h, _ptr(out), count, offset))
        return out

    def mac_write_pairs(self, features: np.ndarray, labels: np.ndarray):
        f = np.ascontiguousarray(features, dtype=np.float32)
        y = np.ascontiguousarray(labels, dtype=np.float32)
        self._chk(lib().gbh_mac_write_pairs(self._h, _ptr(f), _ptr(y), len(y)))

    def mac_train(self, epochs: int, batch: int = 8192, lr: float = 3e-3, seed: int = 0) -> np.ndarray:
        losses = np.zeros(epochs, dtype=np.float32)
        self._chk(lib().gbh_mac_train(self._h, epochs, batch, lr, seed, _ptr(losses)))
        return losses

    def mac_loss_grad(self, features: np.ndarray, labels: np.ndarray):
        f = np.ascontiguousarray(features, dtype=np.float32)
        y = np.ascontiguousarray(labels, dtype=np.float32)
        loss = C.c_float(0)
        grad = np.zeros(abi.MAC_NUM_PARAMS, dtype=np.float32)
        self._chk(lib().gbh_mac_loss_grad(self._h, _ptr(f), _ptr(y), len(y), C.byref(loss), _ptr(grad)))
        return float(loss.value), grad

    def mac_predict(self, features: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(features, dtype=np.float32)
        out = np.zeros(len(f), dtype=np.float32)
        self._chk(lib().gbh_mac_predict(self._h, _ptr(f), len(f), _ptr(out)))
        return out
