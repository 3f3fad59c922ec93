"""Generate the golden vectors in tests/golden/*.npz from the reference harness.

The harness (oracle/ref_glsl, oracle/ref_harness.py) runs the reference's own
GLSL compute kernels compiled as C++; it exists only where the reference
sources are mounted.  Each small fixture (1,024 bodies) stores its input
bodies, bounds, units and step parameters and the reference's outputs, so
tests can check the CPU oracle and the GPU path against the reference
anywhere.  The large fixtures (large_*.npz, 65,536 bodies: 16 tiles of the
GPU sort, about 128 tiles of its fill) store the generator of their inputs
(tests/golden/large_inputs.py) with a digest of the bodies, digests of the
reference's exact outputs, and every 16th body after the step.

view_select.npz holds the outputs of the reference's node-glow and region
vertex shaders (compiled as C++ by oracle/ref_glsl/ref_render.cpp) over the
reference's tree of a 2,048-body Plummer sphere, for three views.

Usage: python tests/golden/make_golden.py [--large-only | --views-only]
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gravity_gb300 import abi, ic  # noqa: E402
from oracle import ref_harness as R  # noqa: E402
from tests.golden import large_inputs as L  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

PARAM_FIELDS = ["dt", "theta", "softening", "elasticity", "restitution", "merging_collision_or_neither",
                "static_or_dynamic", "wrap_around"]


def plummer_with_defects(n, seed):
    b = ic.plummer(n, seed=seed)
    rng = np.random.default_rng(seed + 100)
    dead = rng.choice(n, n // 20, replace=False)
    b["pos_mass"][dead, 3] = 0.0
    b["pos_mass"][rng.choice(n, 2, replace=False), 0] = np.nan
    b["pos_mass"][rng.choice(n, 3, replace=False), :3] *= 50.0
    return b


def live_bounds(b):
    ok = (b["pos_mass"][:, 3] != 0) & np.all(np.isfinite(b["pos_mass"][:, :3]), axis=1)
    p = b["pos_mass"][ok, :3]
    return np.concatenate([p.min(0), p.max(0)]).astype(np.float32)


def cases():
    yield "plummer_dynamic", plummer_with_defects(1024, 11), None, abi.step_params(
        dt=1e-3, theta=0.5, softening=1e-4, bounds=abi.BOUNDS_DYNAMIC), 3
    b = ic.uniform_merge(1024, seed=12)
    b["pos_mass"][:, :3] *= 0.05
    b["pos_mass"][:8, 0] = 3.0
    yield "merge_static", b, np.array([-2, -2, -2, 2, 2, 2], np.float32), abi.step_params(
        dt=5e-4, theta=0.7, softening=1e-8, mode=abi.MODE_MERGE, bounds=abi.BOUNDS_STATIC), 2
    b = ic.uniform_merge(1024, seed=13)
    b["pos_mass"][:, :3] *= 0.05
    b["vel_density"][:, :3] = np.random.default_rng(13).normal(0, 0.1, (1024, 3))
    yield "collision_wrap", b, np.array([-0.05, -0.05, -0.05, 0.05, 0.05, 0.05], np.float32), abi.step_params(
        dt=5e-4, theta=0.7, softening=1e-8, mode=abi.MODE_COLLISION, bounds=abi.BOUNDS_STATIC, wrap=True,
        elasticity=0.5), 2
    b = ic.plummer(1024, seed=14)
    b["pos_mass"][:, :3] = np.random.default_rng(14).integers(0, 3, (1024, 3)).astype(np.float32)
    yield "lattice_duplicates", b, np.array([0, 0, 0, 2, 2, 2], np.float32), abi.step_params(
        dt=1e-3, theta=0.5, softening=1e-2, bounds=abi.BOUNDS_STATIC), 1


LARGE_N = 65536


def large_cases():
    yield "large_clusters_dynamic", ("clusters", LARGE_N, 21), None, abi.step_params(
        dt=1e-3, theta=0.5, softening=1e-4, bounds=abi.BOUNDS_DYNAMIC)
    yield "large_merge_static", ("merge_box", LARGE_N, 22), np.array([-2, -2, -2, 2, 2, 2], np.float32), \
        abi.step_params(dt=5e-4, theta=0.7, softening=1e-8, mode=abi.MODE_MERGE, bounds=abi.BOUNDS_STATIC)


def make_large():
    units = abi.units(G=1.0)
    for name, (kind, n, seed), bounds, p in large_cases():
        bodies = L.make(kind, n, seed)
        if bounds is None:
            bounds = live_bounds(bodies)
        r = R.RefBarnesHut(n, bounds, units)
        r.upload_bodies(bodies)
        r.init()
        r.stage_reset(p)
        r.stage_prepare(p)
        s = r.read_sim_values()
        nl = s.num_bodies
        out = {"kind": np.array(kind), "n": n, "seed": seed, "input_sha256": np.array(L.digest(bodies)),
               "bounds": bounds, "params": np.array([float(getattr(p, f)) for f in PARAM_FIELDS]),
               "prep_num_bodies": nl,
               "prep_bounds": np.array(list(s.bounds_min) + list(s.bounds_max), np.float32),
               "prep_index": np.array(L.digest(r.read_index())),
               "prep_morton": np.array(L.digest(r.read_morton()[:nl]))}
        r.stage_sort()
        r.stage_build()
        r.stage_fill()
        r.stage_walk(p)
        tasks = r.read_merge_tasks()
        out["tasks"] = np.array(L.task_digest(tasks))
        out["task_count"] = len(tasks)
        r.stage_merge(p)
        r.stage_swap()
        out["sorted_index"] = np.array(L.digest(r.read_index()[:nl]))
        out["sorted_morton"] = np.array(L.digest(r.read_morton()[:nl]))
        for f, d in L.node_digests(r.read_internal_nodes()[: max(nl - 1, 1)]).items():
            out[f"internal_{f}"] = np.array(d)
        for f, d in L.node_digests(r.read_leaf_nodes()[:nl]).items():
            out[f"leaf_{f}"] = np.array(d)
        after = r.read_bodies()
        out["bodies_after"] = np.array(L.digest(after.view(np.float32)))
        out["bodies_sample"] = after[::16].copy()
        out["dead_after"] = np.array(L.digest((after["pos_mass"][:, 3] == 0).astype(np.uint8)))
        sv = r.read_sim_values()
        out["uint_debug0"] = sv.uint_debug[0]
        out["out_of_bounds"] = sv.out_of_bounds
        r.close()
        path = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(path, os.path.getsize(path), "tasks", len(tasks))


VIEW_N = 2048


def views():
    """Three cameras over the tree: far and absolute, oblique and absolute,
    near and relative to body 7 (camera scale 1)."""
    fov, aspect = np.radians(50.0), 16.0 / 9.0
    proj = abi.perspective(fov, aspect, 0.01, 1e5)
    out = []
    for eye, rel, scale, depths in [((0, 0, 60), 0xFFFFFFFF, 10.0, (2, 6)),
                                    ((30, 20, 15), 0xFFFFFFFF, 10.0, (0, 3)),
                                    ((5, -4, 8), 7, 1.0, (4, 30))]:
        mv = abi.look_at(eye, (0, 0, 0))
        v = abi.view(mv, proj, fov, aspect, camera_scale=scale, relative_to=rel, glow_max_depth=12,
                     glow_intensity=0.05, region_depths=depths)
        mvp = (np.asarray(proj, np.float64) @ np.asarray(mv, np.float64)).astype(np.float32).T.reshape(-1)
        out.append((v, mvp))
    return out


def make_views():
    """nodeglow.vert and regions.vert of the reference over the tree of a
    2,048-body Plummer sphere built by the reference's kernels, for three
    views: per selected node the shader's outputs and clip positions."""
    import ctypes as C

    n = VIEW_N
    bodies = ic.plummer(n, seed=31)
    bounds = live_bounds(bodies)
    p = abi.step_params(theta=0.5, softening=1e-4)
    r = R.RefBarnesHut(n, bounds, abi.units(G=1.0))
    r.upload_bodies(bodies)
    r.init()
    r.stage_reset(p)
    r.stage_prepare(p)
    r.stage_sort()
    r.stage_build()
    r.stage_fill()
    nodes = r.read_internal_nodes()[: n - 1].copy()
    state = r.read_bodies()
    r.close()
    out = {"bodies": bodies, "bounds": bounds, "params": np.array([float(getattr(p, f)) for f in PARAM_FIELDS])}
    for k, (v, mvp) in enumerate(views()):
        glow, reg = R.render_instances(nodes, state, n, v, mvp)
        gsel = np.nonzero(glow[:, 0, 6] != 0)[0].astype(np.uint32)  # culled instances have vIntensity 0
        culled = (reg[:, 0, 0] == 2) & (reg[:, 0, 1] == 2) & (reg[:, 0, 2] == 2) & (reg[:, 0, 3] == 1)
        rsel = np.nonzero(~culled[: n - 1])[0].astype(np.uint32)  # live nodes [0, n - 1)
        out[f"v{k}_view"] = np.frombuffer(bytes(v), np.uint8)
        out[f"v{k}_mvp"] = mvp
        out[f"v{k}_glow_nodes"] = gsel
        out[f"v{k}_glow_position"] = glow[gsel][:, :, 0:4]        # gl_Position of vertices 0-3
        out[f"v{k}_glow_outputs"] = glow[gsel][:, 0, 6:15]         # vIntensity, vColor, vCenterView, vNdcScale
        out[f"v{k}_region_nodes"] = rsel
        out[f"v{k}_region_position"] = reg[rsel][:, :, 0:4]        # gl_Position at the corners -0.5, +0.5
        out[f"v{k}_region_depth"] = reg[rsel][:, 0, 4].astype(np.uint32)
        print("view", k, "glow", len(gsel), "regions", len(rsel))
    path = os.path.join(OUT, "view_select.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


def main():
    units = abi.units(G=1.0)
    if "--large-only" in sys.argv:
        make_large()
        return
    if "--views-only" in sys.argv:
        make_views()
        return
    make_large()
    make_views()
    for name, bodies, bounds, p, steps in cases():
        if bounds is None:
            bounds = live_bounds(bodies)
        n = len(bodies)
        r = R.RefBarnesHut(n, bounds, units)
        r.upload_bodies(bodies)
        r.init()
        per_step = []
        for _ in range(steps):
            # stage by stage so the first step's intermediate outputs are kept
            r.stage_reset(p)
            r.stage_prepare(p)
            s = r.read_sim_values()
            rec = {"prep_index": r.read_index(), "prep_morton": r.read_morton()[: s.num_bodies].copy(),
                   "prep_bounds": np.array(list(s.bounds_min) + list(s.bounds_max), np.float32),
                   "prep_num_bodies": s.num_bodies}
            r.stage_sort()
            r.stage_build()
            r.stage_fill()
            r.stage_walk(p)
            rec["tasks"] = r.read_merge_tasks()
            r.stage_merge(p)
            r.stage_swap()
            nl = s.num_bodies
            rec.update({
                "sorted_index": r.read_index()[:nl].copy(), "sorted_morton": r.read_morton()[:nl].copy(),
                "internal": r.read_internal_nodes()[: max(nl - 1, 1)].copy(), "leaf": r.read_leaf_nodes()[:nl].copy(),
                "bodies_after": r.read_bodies(), "uint_debug0": r.read_sim_values().uint_debug[0],
                "out_of_bounds": r.read_sim_values().out_of_bounds,
            })
            per_step.append(rec)
        r.close()
        arrays = {"bodies": bodies, "bounds": bounds, "steps": steps,
                  "params": np.array([float(getattr(p, f)) for f in PARAM_FIELDS])}
        for k, rec in enumerate(per_step):
            for key, v in rec.items():
                arrays[f"s{k}_{key}"] = np.asarray(v)
        path = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(path, **arrays)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
