"""The C-ABI library loads and exports every entry point include/gbh.h
declares, and the Python/ctypes struct layouts equal the C header's (checked
with a compiled probe).  No compute call is made (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np

from gravity_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbh.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(gbh_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("gbh_create", "gbh_step", "gbh_init", "gbh_destroy", "gbh_upload_bodies", "gbh_stage_sort",
                 "gbh_read_sim_values", "gbh_last_error", "gbh_direct_sum", "gbh_mac_train"):
        assert must in names


def test_library_exports_every_declared_symbol(gbh_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", gbh_lib._name], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (gbh_\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_abi_version_and_no_device_error(gbh_lib):
    assert gbh_lib.gbh_abi_version() == 1
    h = C.c_void_p()
    b = (C.c_float * 6)(-1, -1, -1, 1, 1, 1)
    u = abi.units()
    rc = gbh_lib.gbh_create(C.byref(h), 0, b, C.byref(u), 0)
    assert rc == abi.GBH_ERR_INVALID  # zero bodies is rejected before any device call
    assert b"initial_num_bodies" in gbh_lib.gbh_last_error(None)
    rc = gbh_lib.gbh_create(None, 16, b, C.byref(u), 0)
    assert rc == abi.GBH_ERR_INVALID


PROBE = r"""
#include <stddef.h>
#include <stdio.h>
#include "gbh.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
int main(void) {
  printf("sizeof.gbh_body %zu\nsizeof.gbh_node %zu\nsizeof.gbh_sim_values %zu\nsizeof.gbh_step_params %zu\n"
         "sizeof.gbh_units %zu\nsizeof.gbh_stats %zu\nsizeof.gbh_device_buffers %zu\n"
         "sizeof.gbh_diagnostics %zu\noffsetof.diag.live_bodies %zu\n",
         sizeof(gbh_body), sizeof(gbh_node), sizeof(gbh_sim_values), sizeof(gbh_step_params),
         sizeof(gbh_units), sizeof(gbh_stats), sizeof(gbh_device_buffers),
         sizeof(gbh_diagnostics), offsetof(gbh_diagnostics, live_bodies));
  P(gbh_node, child_a); P(gbh_node, parent_id); P(gbh_node, avg_color);
  P(gbh_sim_values, bounds_min); P(gbh_sim_values, bounds_max); P(gbh_sim_values, unit_mass);
  P(gbh_sim_values, gravitational_constant); P(gbh_sim_values, uint_debug); P(gbh_sim_values, float_debug);
  P(gbh_step_params, units); P(gbh_step_params, mac_mode); P(gbh_step_params, flags);
  P(gbh_stats, alive); P(gbh_stats, error_word);
  printf("sizeof.gbh_view %zu\nsizeof.gbh_glow_splat %zu\nsizeof.gbh_region %zu\n", sizeof(gbh_view),
         sizeof(gbh_glow_splat), sizeof(gbh_region));
  P(gbh_view, fov_y); P(gbh_view, relative_to); P(gbh_view, glow_intensity); P(gbh_view, region_max_depth);
  P(gbh_glow_splat, intensity); P(gbh_glow_splat, node); P(gbh_glow_splat, ndc_scale); P(gbh_glow_splat, depth);
  P(gbh_region, node); P(gbh_region, depth);
  printf("sizeof.gbh_ic_params %zu\n", sizeof(gbh_ic_params));
  P(gbh_ic_params, center); P(gbh_ic_params, G); P(gbh_ic_params, clusters); P(gbh_ic_params, sigma_hi);
  return 0;
}
"""


def test_struct_layouts_match_header():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(src, "w").write(PROBE)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    got = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    got = {k: int(v) for k, v in got.items()}
    assert got["sizeof.gbh_body"] == abi.BODY_DTYPE.itemsize == 32
    assert got["sizeof.gbh_node"] == abi.NODE_DTYPE.itemsize == 80
    assert got["sizeof.gbh_sim_values"] == C.sizeof(abi.SimValues) == 896
    assert got["sizeof.gbh_step_params"] == C.sizeof(abi.StepParams)
    assert got["sizeof.gbh_units"] == C.sizeof(abi.Units)
    assert got["sizeof.gbh_stats"] == C.sizeof(abi.Stats)
    assert got["sizeof.gbh_diagnostics"] == C.sizeof(abi.Diagnostics)
    assert got["offsetof.diag.live_bodies"] == abi.Diagnostics.live_bodies.offset
    assert got["sizeof.gbh_device_buffers"] == C.sizeof(abi.DeviceBuffers)
    assert got["gbh_node.child_a"] == 40 and got["gbh_node.parent_id"] == 60 and got["gbh_node.avg_color"] == 64
    assert got["gbh_sim_values.bounds_min"] == 32 and got["gbh_sim_values.bounds_max"] == 48
    assert got["gbh_sim_values.unit_mass"] == 64 and got["gbh_sim_values.gravitational_constant"] == 84
    assert got["gbh_sim_values.uint_debug"] == 92 and got["gbh_sim_values.float_debug"] == 492
    assert got["gbh_step_params.units"] == abi.StepParams.units.offset
    assert got["gbh_step_params.mac_mode"] == abi.StepParams.mac_mode.offset
    assert got["gbh_step_params.flags"] == abi.StepParams.flags.offset
    assert got["gbh_stats.alive"] == abi.Stats.alive.offset
    assert got["gbh_stats.error_word"] == abi.Stats.error_word.offset
    assert got["sizeof.gbh_view"] == C.sizeof(abi.View) == 176
    for f in ("fov_y", "relative_to", "glow_intensity", "region_max_depth"):
        assert got[f"gbh_view.{f}"] == getattr(abi.View, f).offset
    assert got["sizeof.gbh_glow_splat"] == abi.GLOW_SPLAT_DTYPE.itemsize
    for f in ("intensity", "node", "ndc_scale", "depth"):
        assert got[f"gbh_glow_splat.{f}"] == abi.GLOW_SPLAT_DTYPE.fields[f][1]
    assert got["sizeof.gbh_ic_params"] == C.sizeof(abi.IcParams) == 144
    for f in ("center", "G", "clusters", "sigma_hi"):
        assert got[f"gbh_ic_params.{f}"] == getattr(abi.IcParams, f).offset
    assert got["sizeof.gbh_region"] == abi.REGION_DTYPE.itemsize
    for f in ("node", "depth"):
        assert got[f"gbh_region.{f}"] == abi.REGION_DTYPE.fields[f][1]


def test_body_layout_is_two_vec4():
    b = np.zeros(2, dtype=abi.BODY_DTYPE)
    b["pos_mass"][1] = [1, 2, 3, 4]
    b["vel_density"][1] = [5, 6, 7, 8]
    assert list(b.view(np.float32)[8:]) == [1, 2, 3, 4, 5, 6, 7, 8]


def test_no_oracle_in_product():
    # the product package and CUDA sources never load the checker
    pkg = os.path.join(ROOT, "gravity_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in text.replace("oracle is", ""), (f, "mentions the oracle")
