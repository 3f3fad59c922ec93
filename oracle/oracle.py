"""ctypes wrapper of the CPU oracle (oracle/_build/libbh_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The product never imports it.

The class mirrors gravity_gb300.BarnesHut (same method names) so a parity test
can drive both with the same call sequence.  Stage methods follow the
reference's own stage boundaries (BarnesHut.java:99-164).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from gravity_gb300 import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libbh_oracle.so")
_lib = None


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    r = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
        L.orc_create.restype = vp
        L.orc_create.argtypes = [u32, C.POINTER(C.c_float), C.POINTER(abi.Units)]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_threads.argtypes = [i32]
        L.orc_get_threads.restype = i32
        sp = C.POINTER(abi.StepParams)
        for name, args in {
            "orc_upload_bodies": [vp, vp, u32, u32],
            "orc_init": [vp],
            "orc_step": [vp, sp],
            "orc_stage_reset": [vp, sp],
            "orc_stage_partition": [vp],
            "orc_stage_decrement": [vp],
            "orc_stage_bounds": [vp],
            "orc_stage_encode": [vp],
            "orc_stage_sort": [vp],
            "orc_stage_build": [vp],
            "orc_stage_fill": [vp],
            "orc_stage_walk": [vp, sp],
            "orc_stage_merge": [vp],
            "orc_stage_swap": [vp],
            "orc_stage_walk_sample": [vp, sp, u32, C.POINTER(u64)],
            "orc_read_bodies": [vp, u32, vp, u32, u32],
            "orc_read_leaf_nodes": [vp, vp, u32, u32],
            "orc_read_internal_nodes": [vp, vp, u32, u32],
            "orc_read_sim_values": [vp, C.POINTER(abi.SimValues)],
            "orc_read_index": [vp, vp, u32, u32],
            "orc_read_morton": [vp, vp, u32, u32],
            "orc_read_merge_tasks": [vp, vp, u32, C.POINTER(u32)],
            "orc_read_accel": [vp, vp, u32, u32],
            "orc_read_stats": [vp, C.POINTER(abi.Stats)],
            "orc_write_sim_values": [vp, C.POINTER(abi.SimValues)],
            "orc_write_index": [vp, vp, u32, u32],
            "orc_write_morton": [vp, vp, u32, u32],
            "orc_direct_sum_fp64": [vp, u32, vp, u32, C.c_double, C.c_double, vp],
            "orc_step_shard_walk": [vp, sp, u32, u32, C.POINTER(u32)],
            "orc_shard_pack": [vp, u32, u32, vp],
            "orc_shard_unpack": [vp, u32, u32, vp],
            "orc_read_merge_tasks_full": [vp, vp, vp, u32, C.POINTER(u32)],
            "orc_write_merge_tasks": [vp, vp, vp, u32],
            "orc_step_shard_finish": [vp, u32],
            "orc_safe_lcp": [vp, i32, i32, i32],
        }.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = i32
        L.orc_expand_bits21.restype = u64
        L.orc_expand_bits21.argtypes = [u32]
        L.orc_morton3d64.restype = u64
        L.orc_morton3d64.argtypes = [u32, u32, u32]
        L.orc_morton_encode.restype = u64
        L.orc_morton_encode.argtypes = [C.POINTER(C.c_float)] * 3
        L.orc_star_color.restype = None
        L.orc_star_color.argtypes = [C.c_float, C.c_float, C.POINTER(C.c_float)]
        for name in ("orc_select_glow_nodes", "orc_select_regions"):
            f = getattr(L, name)
            f.restype = u32
            f.argtypes = [vp, u32, vp, u32, C.POINTER(abi.View), vp, u32]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class OracleBarnesHut:
    """CPU restatement of one simulation context (mirrors gravity_gb300.BarnesHut)."""

    def __init__(self, initial_num_bodies: int, bounds, units: abi.Units | None = None):
        self.n = int(initial_num_bodies)
        b = (C.c_float * 6)(*[float(x) for x in np.asarray(bounds, dtype=np.float32).reshape(-1)])
        self._units = units if units is not None else abi.units()
        self._h = lib().orc_create(self.n, b, C.byref(self._units))
        if not self._h:
            raise RuntimeError("orc_create failed")

    def close(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # lifecycle
    def upload_bodies(self, bodies: np.ndarray, offset: int = 0):
        b = np.ascontiguousarray(bodies, dtype=abi.BODY_DTYPE)
        _check(lib().orc_upload_bodies(self._h, _ptr(b), len(b), offset), "upload_bodies")

    def init(self):
        _check(lib().orc_init(self._h), "init")

    def step(self, params: abi.StepParams):
        _check(lib().orc_step(self._h, C.byref(params)), "step")

    # reference stages
    def stage_reset(self, p):
        _check(lib().orc_stage_reset(self._h, C.byref(p)), "reset")

    def stage_partition(self):
        _check(lib().orc_stage_partition(self._h), "partition")

    def stage_decrement(self):
        _check(lib().orc_stage_decrement(self._h), "decrement")

    def stage_bounds(self):
        _check(lib().orc_stage_bounds(self._h), "bounds")

    def stage_encode(self):
        _check(lib().orc_stage_encode(self._h), "encode")

    def stage_prepare(self, p):
        """partition + decrement + bounds (dynamic) + encode, the GPU's fused stage."""
        self.stage_partition()
        self.stage_decrement()
        if p.static_or_dynamic == abi.BOUNDS_DYNAMIC:
            self.stage_bounds()
        self.stage_encode()

    def stage_sort(self):
        _check(lib().orc_stage_sort(self._h), "sort")

    def stage_build(self):
        _check(lib().orc_stage_build(self._h), "build")

    def stage_fill(self):
        _check(lib().orc_stage_fill(self._h), "fill")

    def stage_walk(self, p):
        _check(lib().orc_stage_walk(self._h, C.byref(p)), "walk")

    def stage_merge(self, p=None):
        _check(lib().orc_stage_merge(self._h), "merge")

    def stage_swap(self):
        _check(lib().orc_stage_swap(self._h), "swap")

    def walk_sample(self, p, stride: int) -> int:
        inter = C.c_uint64(0)
        _check(lib().orc_stage_walk_sample(self._h, C.byref(p), stride, C.byref(inter)), "walk_sample")
        return int(inter.value)

    # the sharded step (same method names as gravity_gb300.BarnesHut); the
    # oracle walks with the plain rule only, so its records are the bodies
    shard_bytes_per_body = abi.BODY_DTYPE.itemsize

    def step_shard_walk(self, p, rank: int, world: int) -> tuple[int, int]:
        r = (C.c_uint32 * 2)()
        _check(lib().orc_step_shard_walk(self._h, C.byref(p), rank, world, r), "step_shard_walk")
        return int(r[0]), int(r[1])

    def shard_pack_tensor(self, lo: int, hi: int):
        import torch

        out = np.zeros(hi - lo, dtype=abi.BODY_DTYPE)
        _check(lib().orc_shard_pack(self._h, lo, hi - lo, _ptr(out)), "shard_pack")
        return torch.from_numpy(out.view(np.uint8).copy())

    def shard_unpack_tensor(self, lo: int, t):
        a = np.ascontiguousarray(t.cpu().numpy()).view(abi.BODY_DTYPE)
        _check(lib().orc_shard_unpack(self._h, lo, len(a), _ptr(a)), "shard_unpack")

    def read_merge_tasks_full(self):
        cnt = C.c_uint32(0)
        _check(lib().orc_read_merge_tasks_full(self._h, None, None, 0, C.byref(cnt)), "read_merge_tasks_full")
        pairs = np.zeros((cnt.value, 2), np.uint32)
        keys = np.zeros(cnt.value, np.uint64)
        if cnt.value:
            _check(lib().orc_read_merge_tasks_full(self._h, _ptr(pairs), _ptr(keys), cnt.value, C.byref(cnt)),
                   "read_merge_tasks_full")
        return pairs, keys, np.zeros(cnt.value, np.uint32)

    def write_merge_tasks(self, pairs, keys, slots):
        p = np.ascontiguousarray(pairs, np.uint32)
        k = np.ascontiguousarray(keys, np.uint64)
        _check(lib().orc_write_merge_tasks(self._h, _ptr(p), _ptr(k), len(k)), "write_merge_tasks")

    def step_shard_finish(self, out_of_bounds_other_ranks: int):
        _check(lib().orc_step_shard_finish(self._h, out_of_bounds_other_ranks), "step_shard_finish")

    # read-back
    def read_bodies(self, which=abi.BODIES_IN, count=None, offset=0) -> np.ndarray:
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=abi.BODY_DTYPE)
        _check(lib().orc_read_bodies(self._h, which, _ptr(out), count, offset), "read_bodies")
        return out

    def read_leaf_nodes(self, count=None, offset=0) -> np.ndarray:
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=abi.NODE_DTYPE)
        _check(lib().orc_read_leaf_nodes(self._h, _ptr(out), count, offset), "read_leaf_nodes")
        return out

    def read_internal_nodes(self, count=None, offset=0) -> np.ndarray:
        cap = max(self.n - 1, 1)
        count = cap - offset if count is None else count
        out = np.zeros(count, dtype=abi.NODE_DTYPE)
        _check(lib().orc_read_internal_nodes(self._h, _ptr(out), count, offset), "read_internal_nodes")
        return out

    def read_sim_values(self) -> abi.SimValues:
        s = abi.SimValues()
        _check(lib().orc_read_sim_values(self._h, C.byref(s)), "read_sim_values")
        return s

    def read_index(self, count=None, offset=0) -> np.ndarray:
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=np.uint32)
        _check(lib().orc_read_index(self._h, _ptr(out), count, offset), "read_index")
        return out

    def read_morton(self, count=None, offset=0) -> np.ndarray:
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=np.uint64)
        _check(lib().orc_read_morton(self._h, _ptr(out), count, offset), "read_morton")
        return out

    def read_merge_tasks(self) -> np.ndarray:
        cnt = C.c_uint32(0)
        _check(lib().orc_read_merge_tasks(self._h, None, 0, C.byref(cnt)), "read_merge_tasks")
        out = np.zeros((cnt.value, 2), dtype=np.uint32)
        if cnt.value:
            _check(lib().orc_read_merge_tasks(self._h, _ptr(out), cnt.value, C.byref(cnt)), "read_merge_tasks")
        return out

    def read_accel(self, count=None, offset=0) -> np.ndarray:
        count = self.n - offset if count is None else count
        out = np.zeros((count, 4), dtype=np.float32)
        _check(lib().orc_read_accel(self._h, _ptr(out), count, offset), "read_accel")
        return out

    def read_stats(self) -> abi.Stats:
        s = abi.Stats()
        _check(lib().orc_read_stats(self._h, C.byref(s)), "read_stats")
        return s

    def write_sim_values(self, s: abi.SimValues):
        _check(lib().orc_write_sim_values(self._h, C.byref(s)), "write_sim_values")

    def write_index(self, idx: np.ndarray, offset=0):
        a = np.ascontiguousarray(idx, dtype=np.uint32)
        _check(lib().orc_write_index(self._h, _ptr(a), len(a), offset), "write_index")

    def write_morton(self, keys: np.ndarray, offset=0):
        a = np.ascontiguousarray(keys, dtype=np.uint64)
        _check(lib().orc_write_morton(self._h, _ptr(a), len(a), offset), "write_morton")


def direct_sum_fp64(bodies: np.ndarray, sample: np.ndarray, G: float, softening: float) -> np.ndarray:
    b = np.ascontiguousarray(bodies, dtype=abi.BODY_DTYPE)
    s = np.ascontiguousarray(sample, dtype=np.uint32)
    out = np.zeros((len(s), 3), dtype=np.float64)
    _check(lib().orc_direct_sum_fp64(_ptr(b), len(b), _ptr(s), len(s), G, softening, _ptr(out)), "direct_sum")
    return out


def _select(fn, internal: np.ndarray, bodies: np.ndarray, view: abi.View, dtype: np.dtype):
    nodes = np.ascontiguousarray(internal, dtype=abi.NODE_DTYPE)
    b = np.ascontiguousarray(bodies, dtype=abi.BODY_DTYPE)
    out = np.zeros(max(len(nodes), 1), dtype=dtype)
    sel = fn(_ptr(nodes), len(nodes), _ptr(b), len(b), C.byref(view), _ptr(out), len(out))
    return out[:min(sel, len(out))], int(sel)


def select_glow_nodes(internal: np.ndarray, bodies: np.ndarray, view: abi.View):
    """(records in node order, selected) of nodeglow.vert over the live internal nodes."""
    return _select(lib().orc_select_glow_nodes, internal, bodies, view, abi.GLOW_SPLAT_DTYPE)


def select_regions(internal: np.ndarray, bodies: np.ndarray, view: abi.View):
    """(records in node order, selected) of regions.vert over the live internal nodes."""
    return _select(lib().orc_select_regions, internal, bodies, view, abi.REGION_DTYPE)


def morton_encode(pos, bmin, bmax) -> int:
    f3 = C.c_float * 3
    return int(lib().orc_morton_encode(f3(*pos), f3(*bmin), f3(*bmax)))


def morton3d64(x: int, y: int, z: int) -> int:
    return int(lib().orc_morton3d64(x, y, z))


def safe_lcp(keys: np.ndarray, i: int, j: int) -> int:
    k = np.ascontiguousarray(keys, dtype=np.uint64)
    return int(lib().orc_safe_lcp(_ptr(k), len(k), i, j))


def star_color(mass: float, density: float) -> np.ndarray:
    out = (C.c_float * 3)()
    lib().orc_star_color(mass, density, out)
    return np.array(list(out), dtype=np.float32)
