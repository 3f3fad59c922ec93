"""gravity_gb300 — GB300-native per-step Barnes–Hut pipeline.

A drop-in for the step of the gkane1234/gravity simulator: the C ABI in
include/gbh.h (libgbh.so, hand-written sm_103a kernels) and this Python host
mirror of the reference's BarnesHut interface.
"""
from . import abi, ic  # noqa: F401
from ._lib import GbhError, LIB_PATH  # noqa: F401
from .barnes_hut import BarnesHut  # noqa: F401
