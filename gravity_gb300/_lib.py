"""Loader of libgbh.so (the in-tree C-ABI library, include/gbh.h) via ctypes.

There is no fallback: if the library is missing or cannot be loaded, every
entry point raises.  Build it with gravity_gb300.build.build().
"""
from __future__ import annotations

import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbh.so")
_lib = None


class GbhError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gbh error {code}: {msg}")
        self.code = code


def _declare(L):
    vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
    sp = C.POINTER(abi.StepParams)
    sigs = {
        "gbh_create": [C.POINTER(vp), u32, C.POINTER(C.c_float), C.POINTER(abi.Units), i32],
        "gbh_destroy": [vp],
        "gbh_upload_bodies": [vp, vp, u32, u32],
        "gbh_init": [vp],
        "gbh_step": [vp, sp],
        "gbh_step_n": [vp, sp, u32],
        "gbh_synchronize": [vp],
        "gbh_clear_error": [vp],
        "gbh_read_bodies": [vp, u32, vp, u32, u32],
        "gbh_read_leaf_nodes": [vp, vp, u32, u32],
        "gbh_read_internal_nodes": [vp, vp, u32, u32],
        "gbh_read_sim_values": [vp, C.POINTER(abi.SimValues)],
        "gbh_read_index": [vp, vp, u32, u32],
        "gbh_read_morton": [vp, vp, u32, u32],
        "gbh_read_merge_tasks": [vp, vp, u32, C.POINTER(u32)],
        "gbh_read_accel": [vp, vp, u32, u32],
        "gbh_read_stats": [vp, C.POINTER(abi.Stats)],
        "gbh_read_potential": [vp, vp, u32, u32],
        "gbh_read_positions_fp64": [vp, vp, u32, u32],
        "gbh_write_positions_fp64": [vp, vp, u32, u32],
        "gbh_read_diagnostics": [vp, C.POINTER(abi.Diagnostics)],
        "gbh_device_ptrs": [vp, C.POINTER(abi.DeviceBuffers)],
        "gbh_write_sim_values": [vp, C.POINTER(abi.SimValues)],
        "gbh_write_index": [vp, vp, u32, u32],
        "gbh_write_morton": [vp, vp, u32, u32],
        "gbh_stage_reset": [vp, sp],
        "gbh_stage_prepare": [vp, sp],
        "gbh_stage_sort": [vp],
        "gbh_stage_build": [vp],
        "gbh_stage_fill": [vp],
        "gbh_stage_walk": [vp, sp],
        "gbh_stage_merge": [vp, sp],
        "gbh_stage_swap": [vp],
        "gbh_step_profiled": [vp, sp, C.POINTER(C.c_float)],
        "gbh_direct_sum": [vp, sp, vp, u32, vp],
        "gbh_mac_set_weights": [vp, vp, u32],
        "gbh_mac_get_weights": [vp, vp, u32],
        "gbh_mac_set_band": [vp, C.c_float, C.c_float],
        "gbh_mac_get_band": [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)],
        "gbh_mac_generate": [vp, sp, u32, u64, C.POINTER(u32)],
        "gbh_mac_read_pairs": [vp, vp, vp, u32, u32],
        "gbh_mac_write_pairs": [vp, vp, vp, u32],
        "gbh_mac_read_pair_ids": [vp, vp, u32, u32],
        "gbh_mac_train": [vp, u32, u32, C.c_float, u64, vp],
        "gbh_mac_loss_grad": [vp, vp, vp, u32, C.POINTER(C.c_float), vp],
        "gbh_mac_predict": [vp, vp, u32, vp],
        "gbh_sort_pairs_noalloc": [vp, vp, vp, vp, u32, vp],
        "gbh_exchange_bodies": [vp, vp, vp, u32, u32],
        "gbh_step_streamed": [vp, sp, vp, vp],
        "gbh_step_shard_walk": [vp, sp, u32, u32, C.POINTER(u32)],
        "gbh_shard_pack": [vp, u32, u32, vp],
        "gbh_shard_unpack": [vp, u32, u32, vp],
        "gbh_read_merge_tasks_full": [vp, vp, vp, vp, u32, C.POINTER(u32)],
        "gbh_write_merge_tasks": [vp, vp, vp, vp, u32],
        "gbh_step_shard_finish": [vp, u32],
        "gbh_step_streamed_finish": [vp, vp],
        "gbh_generate_bodies": [vp, C.POINTER(abi.IcParams), u64, u32, u32],
        "gbh_select_glow_nodes": [vp, C.POINTER(abi.View), vp, u32, C.POINTER(u32)],
        "gbh_select_regions": [vp, C.POINTER(abi.View), vp, u32, C.POINTER(u32)],
    }
    for name, args in sigs.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = i32
    L.gbh_abi_version.argtypes = []
    L.gbh_abi_version.restype = i32
    L.gbh_last_error.argtypes = [vp]
    L.gbh_last_error.restype = C.c_char_p
    L.gbh_stream.argtypes = [vp]
    L.gbh_stream.restype = vp
    return L


def lib():
    """The loaded library; raises if libgbh.so is absent (no fallback path)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise GbhError(abi.GBH_ERR_UNSUPPORTED, f"{LIB_PATH} is missing: run gravity_gb300.build.build()")
        _lib = _declare(C.CDLL(LIB_PATH))
        if _lib.gbh_abi_version() != 1:
            raise GbhError(abi.GBH_ERR_UNSUPPORTED, "libgbh.so ABI version mismatch")
    return _lib


def check(rc: int, handle=None) -> None:
    if rc != 0:
        msg = lib().gbh_last_error(handle)
        raise GbhError(rc, msg.decode() if msg else "")
