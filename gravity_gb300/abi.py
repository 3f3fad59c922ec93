"""ctypes / numpy mirrors of the structs declared in include/gbh.h.

The layouts are the reference's std430 SSBO layouts
(src/main/resources/shaders/common/common.glsl:25-120): Body 32 bytes, Node 80
bytes, SimulationValues 896 bytes.  Module-level asserts pin every offset.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

# status codes
GBH_OK = 0
GBH_ERR_INVALID = -1
GBH_ERR_CUDA = -2
GBH_ERR_OOM = -3
GBH_ERR_DEVICE = -4
GBH_ERR_STATE = -5
GBH_ERR_UNSUPPORTED = -6

# device error word bits
DEVERR_SORT_LOOKBACK = 0x1
DEVERR_FILL_SPIN = 0x2
DEVERR_WALK_STACK = 0x4
DEVERR_MERGE_OVERFLOW = 0x8
DEVERR_TREE_HEIGHT = 0x10
DEVERR_MAC_FRONTIER = 0x20

# mergingCollisionOrNeither / staticOrDynamic (common.glsl:133-149)
MODE_NEITHER, MODE_MERGE, MODE_COLLISION = 0, 1, 2
BOUNDS_STATIC, BOUNDS_DYNAMIC = 0, 1
MAC_PLAIN, MAC_LEARNED, MAC_GROUP = 0, 1, 2
PRECISION_FP32, PRECISION_COMPENSATED = 0, 1
FLAG_STORE_ACCEL = 0x1
FLAG_STORE_POTENTIAL = 0x2
BODIES_IN, BODIES_OUT = 0, 1
NUM_STAGES = 8
STAGE_NAMES = ("reset", "prepare", "sort", "build", "fill", "walk", "merge", "swap")
MAC_FEATURES = 12
MAC_HIDDEN = 32
MAC_NUM_PARAMS = 32 * 12 + 32 + 32 * 32 + 32 + 32 + 1
NONE_ID = 0xFFFFFFFF
SORT_NOALLOC_MAX_PAIRS = 1 << 20  # GBH_SORT_NOALLOC_MAX_PAIRS
SHARD_BYTES_PER_BODY = 36  # GBH_SHARD_BYTES_PER_BODY

BODY_DTYPE = np.dtype([("pos_mass", "<f4", (4,)), ("vel_density", "<f4", (4,))])
NODE_DTYPE = np.dtype(
    [
        ("com_mass", "<f4", (4,)),
        ("aabb", "<f4", (6,)),
        ("child_a", "<u4"),
        ("child_b", "<u4"),
        ("node_depth", "<u4"),
        ("bodies_contained", "<u4"),
        ("ready_children", "<u4"),
        ("parent_id", "<u4"),
        ("avg_color", "<f4", (4,)),
    ]
)
assert BODY_DTYPE.itemsize == 32
assert NODE_DTYPE.itemsize == 80
assert NODE_DTYPE.fields["child_a"][1] == 40
assert NODE_DTYPE.fields["parent_id"][1] == 60
assert NODE_DTYPE.fields["avg_color"][1] == 64


class Units(C.Structure):
    _fields_ = [
        ("mass", C.c_float),
        ("density", C.c_float),
        ("len", C.c_float),
        ("time", C.c_float),
        ("camera_scale", C.c_float),
        ("gravitational_constant", C.c_float),
    ]


class StepParams(C.Structure):
    _fields_ = [
        ("dt", C.c_float),
        ("theta", C.c_float),
        ("softening", C.c_float),
        ("elasticity", C.c_float),
        ("restitution", C.c_float),
        ("merging_collision_or_neither", C.c_uint32),
        ("static_or_dynamic", C.c_uint32),
        ("wrap_around", C.c_uint32),
        ("units", Units),
        ("mac_mode", C.c_uint32),
        ("precision_mode", C.c_uint32),
        ("mac_tolerance", C.c_float),
        ("flags", C.c_uint32),
    ]


class SimValues(C.Structure):
    _fields_ = [
        ("num_bodies", C.c_uint32),
        ("initial_num_bodies", C.c_uint32),
        ("just_died", C.c_uint32),
        ("merged", C.c_uint32),
        ("out_of_bounds", C.c_uint32),
        ("relative_to", C.c_uint32),
        ("pad1", C.c_uint32),
        ("pad2", C.c_uint32),
        ("bounds_min", C.c_float * 3),
        ("pad_min", C.c_uint32),
        ("bounds_max", C.c_float * 3),
        ("pad_max", C.c_uint32),
        ("unit_mass", C.c_float),
        ("unit_density", C.c_float),
        ("unit_len", C.c_float),
        ("unit_time", C.c_float),
        ("camera_scale", C.c_float),
        ("gravitational_constant", C.c_float),
        ("body_length_constant", C.c_float),
        ("uint_debug", C.c_uint32 * 100),
        ("float_debug", C.c_float * 100),
        ("tail_pad", C.c_uint32),
    ]


assert C.sizeof(SimValues) == 896
assert SimValues.bounds_min.offset == 32
assert SimValues.bounds_max.offset == 48
assert SimValues.unit_mass.offset == 64
assert SimValues.uint_debug.offset == 92
assert SimValues.float_debug.offset == 492


class Stats(C.Structure):
    _fields_ = [
        ("interactions", C.c_uint64),
        ("nodes_opened", C.c_uint64),
        ("mac_evaluations", C.c_uint64),
        ("alive", C.c_uint32),
        ("died", C.c_uint32),
        ("merged", C.c_uint32),
        ("merge_tasks", C.c_uint32),
        ("merge_conflicts", C.c_uint32),
        ("out_of_bounds", C.c_uint32),
        ("tree_height", C.c_uint32),
        ("max_stack", C.c_uint32),
        ("error_word", C.c_uint32),
        ("frontier_saturated", C.c_uint32),
    ]


class Diagnostics(C.Structure):
    """gbh_diagnostics: conserved quantities summed in FP64."""

    _fields_ = [
        ("mass", C.c_double),
        ("momentum", C.c_double * 3),
        ("centre_of_mass", C.c_double * 3),
        ("kinetic_energy", C.c_double),
        ("potential_energy", C.c_double),
        ("total_energy", C.c_double),
        ("angular_momentum", C.c_double * 3),
        ("live_bodies", C.c_uint32),
        ("potential_valid", C.c_uint32),
        ("positions_fp64", C.c_uint32),
        ("pad", C.c_uint32),
    ]


assert C.sizeof(Diagnostics) == 13 * 8 + 16


class DeviceBuffers(C.Structure):
    _fields_ = [
        ("bodies_in", C.c_void_p),
        ("bodies_out", C.c_void_p),
        ("leaf_nodes", C.c_void_p),
        ("internal_nodes", C.c_void_p),
        ("sim_values", C.c_void_p),
        ("morton_in", C.c_void_p),
        ("index_in", C.c_void_p),
        ("merge_tasks", C.c_void_p),
    ]


IC_BOX, IC_DISK, IC_PLUMMER, IC_CLUSTERS = 0, 1, 2, 3
IC_ORBITAL, IC_CCW = 0x1, 0x2


class IcParams(C.Structure):
    """gbh_ic_params: seeded initial conditions generated on the device."""
    _fields_ = [
        ("kind", C.c_uint32),
        ("flags", C.c_uint32),
        ("lo", C.c_float * 8),
        ("hi", C.c_float * 8),
        ("center", C.c_float * 3),
        ("velocity", C.c_float * 3),
        ("scale", C.c_float),
        ("total_mass", C.c_float),
        ("density", C.c_float),
        ("G", C.c_float),
        ("phi", C.c_float),
        ("center_mass", C.c_float),
        ("center_density", C.c_float),
        ("adherence", C.c_float),
        ("orbital_factor", C.c_float),
        ("clusters", C.c_uint32),
        ("sigma_lo", C.c_float),
        ("sigma_hi", C.c_float),
    ]


assert C.sizeof(IcParams) == 144


def ic_params(kind, **kw) -> IcParams:
    """IcParams of `kind` with fields from keywords; `ranges` = 8 (lo, hi)
    pairs for x, y, z, vx, vy, vz, mass, density."""
    p = IcParams()
    p.kind = kind
    p.density, p.G, p.scale, p.total_mass = 1.0, 1.0, 1.0, 1.0
    ranges = kw.pop("ranges", None)
    if ranges is not None:
        for k, (lo, hi) in enumerate(ranges):
            p.lo[k], p.hi[k] = lo, hi
    known = {f for f, _ in IcParams._fields_}
    for name, val in kw.items():
        if name not in known:
            raise TypeError(f"gbh_ic_params has no field {name!r}")
        if name in ("center", "velocity"):
            getattr(p, name)[:] = list(val)
        else:
            setattr(p, name, val)
    return p


class View(C.Structure):
    """gbh_view: the render uniforms of the node glow and region shaders."""
    _fields_ = [
        ("model_view", C.c_float * 16),
        ("proj", C.c_float * 16),
        ("fov_y", C.c_float),
        ("aspect", C.c_float),
        ("camera_scale", C.c_float),
        ("relative_to", C.c_uint32),
        ("glow_theta_ndc", C.c_float),
        ("glow_activate_dist", C.c_float),
        ("glow_max_depth", C.c_int32),
        ("glow_intensity", C.c_float),
        ("region_min_depth", C.c_int32),
        ("region_max_depth", C.c_int32),
        ("pad", C.c_uint32 * 2),
    ]


assert C.sizeof(View) == 176

GLOW_SPLAT_DTYPE = np.dtype([
    ("center_clip", "<f4", (4,)), ("center_view", "<f4", (3,)), ("intensity", "<f4"), ("color", "<f4", (3,)),
    ("node", "<u4"), ("ndc_scale", "<f4", (2,)), ("depth", "<u4"), ("pad", "<u4"),
])
REGION_DTYPE = np.dtype([("center", "<f4", (3,)), ("size", "<f4", (3,)), ("node", "<u4"), ("depth", "<u4")])
assert GLOW_SPLAT_DTYPE.itemsize == 64 and REGION_DTYPE.itemsize == 32


def view(model_view, proj, fov_y, aspect, camera_scale=10.0, relative_to=0xFFFFFFFF, glow_theta_px=16.0,
         height=1080, glow_activate_dist=0.0, glow_max_depth=8, glow_intensity=0.003, region_depths=(0, 8)) -> View:
    """A View from 4x4 matrices (row-major numpy, as written on paper; stored
    column-major like GLSL) and the reference's Settings defaults
    (nodeGlowThetaPx 16, nodeGlowActivateDist 0, nodeGlowMaxDepth 8,
    nodeGlowIntensity 0.003; uNodeGlowThetaNdc = 2 px / height, GPU.java:913-915)."""
    v = View()
    mv = np.asarray(model_view, dtype=np.float32).T.reshape(-1)
    pr = np.asarray(proj, dtype=np.float32).T.reshape(-1)
    v.model_view[:] = mv.tolist()
    v.proj[:] = pr.tolist()
    v.fov_y, v.aspect, v.camera_scale = fov_y, aspect, camera_scale
    v.relative_to = relative_to
    v.glow_theta_ndc = np.float32(2.0) * np.float32(glow_theta_px) / np.float32(max(1.0, height))
    v.glow_activate_dist, v.glow_max_depth, v.glow_intensity = glow_activate_dist, glow_max_depth, glow_intensity
    v.region_min_depth, v.region_max_depth = region_depths
    return v


def look_at(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Row-major 4x4 view matrix (right-handed, camera looking down -z)."""
    eye, target, up = (np.asarray(x, dtype=np.float64) for x in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m.astype(np.float32)


def perspective(fov_y, aspect, near, far) -> np.ndarray:
    """Row-major 4x4 OpenGL perspective projection."""
    t = 1.0 / np.tan(0.5 * fov_y)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = t / aspect, t
    m[2, 2], m[2, 3] = (far + near) / (near - far), 2 * far * near / (near - far)
    m[3, 2] = -1.0
    return m.astype(np.float32)


def units(mass=1.0, density=1.0, length=1.0, time=1.0, camera_scale=10.0, G=0.0) -> Units:
    """UnitSet with the reference defaults (defaultProperties.json: 1,1,1,1, cameraScale 10)."""
    return Units(mass, density, length, time, camera_scale, G)


def step_params(
    dt=1e-3,
    theta=0.5,
    softening=1e-4,
    mode=MODE_NEITHER,
    bounds=BOUNDS_DYNAMIC,
    wrap=False,
    elasticity=1.0,
    restitution=0.2,
    mac=MAC_PLAIN,
    precision=PRECISION_FP32,
    mac_tolerance=-3.0,
    flags=0,
    units_update: Units | None = None,
) -> StepParams:
    """Step uniforms; defaults keep the current units (units.mass == 0)."""
    u = units_update if units_update is not None else Units(0, 0, 0, 0, 0, 0)
    return StepParams(
        dt, theta, softening, elasticity, restitution, mode, bounds, int(bool(wrap)), u, mac, precision,
        mac_tolerance, flags,
    )


def diagnostics_to_dict(d: Diagnostics) -> dict:
    out = {}
    for name, _ in Diagnostics._fields_:
        if name == "pad":
            continue
        v = getattr(d, name)
        out[name] = list(v) if isinstance(v, C.Array) else v
    return out


def sim_to_dict(s: SimValues) -> dict:
    out = {}
    for name, _ in SimValues._fields_:
        v = getattr(s, name)
        if isinstance(v, C.Array):
            v = list(v)
        out[name] = v
    return out


def stats_to_dict(s: Stats) -> dict:
    return {name: getattr(s, name) for name, _ in Stats._fields_}
