"""ctypes wrapper of the reference harness (oracle/_ref/libbh_ref.so).

TEST INFRASTRUCTURE ONLY.  The harness is the reference's own GLSL compute
kernels (src/main/resources/shaders/compute/*/bh_*.comp) compiled as C++ under
oracle/ref_glsl/glsl_shim.hpp and driven like BarnesHut.step.  It is built
only where the reference sources are mounted (the development container), by
oracle/ref_glsl/Makefile, into oracle/_ref/.  It pins the C oracle: the
tests compare the two, and tests/golden/make_golden.py stores its outputs as
golden vectors that the oracle and the GPU path are checked against anywhere.

The harness keeps one global simulation state (one instance at a time).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from gravity_gb300 import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libbh_ref.so")
# the reference checkout: GBH_REFERENCE (default: where this container mounts it)
REF_ROOT = os.environ.get("GBH_REFERENCE", "/root/reference")
REF_SHADERS = os.path.join(REF_ROOT, "src", "main", "resources", "shaders")
_lib = None


RENDER_LIB_PATH = os.path.join(_HERE, "_ref", "libbh_ref_render.so")
_render = None


def render_lib():
    """The reference's node-glow and region vertex shaders compiled as C++
    (oracle/ref_glsl/ref_render.cpp)."""
    global _render
    if _render is None:
        if not os.path.exists(RENDER_LIB_PATH):
            build_if_available()
        L = C.CDLL(RENDER_LIB_PATH)
        L.ref_render_set.restype = None
        L.ref_render_set.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(abi.View),
                                     C.POINTER(C.c_float)]
        for f in (L.ref_glow_instances, L.ref_region_instances):
            f.restype = None
            f.argtypes = [C.c_int, C.c_void_p]
        _render = L
    return _render


def render_instances(internal: np.ndarray, bodies: np.ndarray, num_bodies: int, view, mvp16) -> tuple:
    """Run nodeglow.vert (4 vertices) and regions.vert (2 cube corners) for
    every instance the shaders visit: glow instances [0, len(bodies) - 1),
    region instances [0, num_bodies).  `internal` is padded with zeroed slots
    up to num_bodies (the region shader reads one slot past the live nodes).
    Returns (glow[count][4][16], regions[num_bodies][2][5])."""
    L = render_lib()
    n_cap = len(bodies)
    nodes = np.zeros(max(n_cap, num_bodies) + 1, dtype=abi.NODE_DTYPE)
    nodes[: len(internal)] = internal
    b = np.ascontiguousarray(bodies, dtype=abi.BODY_DTYPE)
    m = (C.c_float * 16)(*[float(x) for x in np.asarray(mvp16, np.float32).reshape(-1)])
    L.ref_render_set(nodes.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p), num_bodies, n_cap,
                     C.byref(view), m)
    glow = np.zeros((n_cap - 1, 4, 16), np.float32)
    L.ref_glow_instances(n_cap - 1, glow.ctypes.data_as(C.c_void_p))
    reg = np.zeros((num_bodies, 2, 5), np.float32)
    L.ref_region_instances(num_bodies, reg.ctypes.data_as(C.c_void_p))
    return glow, reg


def available() -> bool:
    return os.path.exists(LIB_PATH) or os.path.isdir(REF_SHADERS)


def build_if_available() -> str | None:
    if not os.path.isdir(REF_SHADERS):
        return LIB_PATH if os.path.exists(LIB_PATH) else None
    r = subprocess.run(["make", "-C", os.path.join(_HERE, "ref_glsl"), f"REF_SHADERS={REF_SHADERS}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference harness build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


class RefParams(C.Structure):
    _fields_ = [
        ("dt", C.c_float),
        ("theta", C.c_float),
        ("softening", C.c_float),
        ("elasticity", C.c_float),
        ("restitution", C.c_float),
        ("mode", C.c_uint32),
        ("static_or_dynamic", C.c_uint32),
        ("wrap_around", C.c_uint32),
        ("mass", C.c_float),
        ("density", C.c_float),
        ("len", C.c_float),
        ("time", C.c_float),
        ("camera_scale", C.c_float),
        ("G", C.c_float),
    ]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build_if_available()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("reference harness unavailable (reference sources not mounted)")
        L = C.CDLL(LIB_PATH)
        vp, u32, f = C.c_void_p, C.c_uint32, C.c_float
        rp = C.POINTER(RefParams)
        for name, args in {
            "ref_create": [u32, C.POINTER(f), f, f, f, f, f, f],
            "ref_upload_bodies": [vp, u32, u32],
            "ref_init": [],
            "ref_step": [rp],
            "ref_stage_reset": [rp],
            "ref_stage_partition": [],
            "ref_stage_bounds": [],
            "ref_stage_encode": [],
            "ref_stage_sort": [],
            "ref_stage_build": [],
            "ref_stage_fill": [],
            "ref_stage_walk": [rp],
            "ref_stage_merge": [],
            "ref_stage_swap": [],
            "ref_read_bodies": [u32, vp, u32, u32],
            "ref_read_leaf_nodes": [vp, u32, u32],
            "ref_read_internal_nodes": [vp, u32, u32],
            "ref_read_index": [vp, u32, u32],
            "ref_read_morton": [vp, u32, u32],
            "ref_read_sim_values": [vp],
            "ref_read_merge_tasks": [vp, u32, C.POINTER(u32)],
            "ref_write_index": [vp, u32, u32],
            "ref_write_morton": [vp, u32, u32],
        }.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        L.ref_destroy.argtypes = []
        L.ref_destroy.restype = None
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class RefBarnesHut:
    """The reference kernels on the CPU, with the oracle's method names."""

    def __init__(self, initial_num_bodies: int, bounds, units: abi.Units | None = None):
        self.n = int(initial_num_bodies)
        u = units if units is not None else abi.units()
        self.units = u
        b = (C.c_float * 6)(*[float(x) for x in np.asarray(bounds, np.float32).reshape(-1)])
        lib().ref_create(self.n, b, u.mass, u.density, u.len, u.time, u.camera_scale, u.gravitational_constant)

    def close(self):
        lib().ref_destroy()

    def _rp(self, p: abi.StepParams) -> RefParams:
        u = self.units
        return RefParams(p.dt, p.theta, p.softening, p.elasticity, p.restitution, p.merging_collision_or_neither,
                         p.static_or_dynamic, p.wrap_around, u.mass, u.density, u.len, u.time, u.camera_scale,
                         u.gravitational_constant)

    def upload_bodies(self, bodies, offset=0):
        b = np.ascontiguousarray(bodies, dtype=abi.BODY_DTYPE)
        lib().ref_upload_bodies(_ptr(b), len(b), offset)

    def init(self):
        lib().ref_init()

    def step(self, p):
        lib().ref_step(C.byref(self._rp(p)))

    def stage_reset(self, p):
        lib().ref_stage_reset(C.byref(self._rp(p)))

    def stage_prepare(self, p):
        lib().ref_stage_partition()
        if p.static_or_dynamic == abi.BOUNDS_DYNAMIC:
            lib().ref_stage_bounds()
        lib().ref_stage_encode()

    def stage_sort(self):
        lib().ref_stage_sort()

    def stage_build(self):
        lib().ref_stage_build()

    def stage_fill(self):
        lib().ref_stage_fill()

    def stage_walk(self, p):
        lib().ref_stage_walk(C.byref(self._rp(p)))

    def stage_merge(self, p=None):
        lib().ref_stage_merge()

    def stage_swap(self):
        lib().ref_stage_swap()

    def read_bodies(self, which=abi.BODIES_IN, count=None, offset=0):
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=abi.BODY_DTYPE)
        lib().ref_read_bodies(which, _ptr(out), count, offset)
        return out

    def read_leaf_nodes(self, count=None, offset=0):
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=abi.NODE_DTYPE)
        lib().ref_read_leaf_nodes(_ptr(out), count, offset)
        return out

    def read_internal_nodes(self, count=None, offset=0):
        count = max(self.n - 1, 1) - offset if count is None else count
        out = np.zeros(count, dtype=abi.NODE_DTYPE)
        lib().ref_read_internal_nodes(_ptr(out), count, offset)
        return out

    def read_index(self, count=None, offset=0):
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=np.uint32)
        lib().ref_read_index(_ptr(out), count, offset)
        return out

    def read_morton(self, count=None, offset=0):
        count = self.n - offset if count is None else count
        out = np.zeros(count, dtype=np.uint64)
        lib().ref_read_morton(_ptr(out), count, offset)
        return out

    def read_sim_values(self) -> abi.SimValues:
        s = abi.SimValues()
        lib().ref_read_sim_values(C.byref(s))
        return s

    def read_merge_tasks(self):
        cnt = C.c_uint32(0)
        lib().ref_read_merge_tasks(None, 0, C.byref(cnt))
        out = np.zeros((cnt.value, 2), dtype=np.uint32)
        if cnt.value:
            lib().ref_read_merge_tasks(_ptr(out), cnt.value, C.byref(cnt))
        return out
