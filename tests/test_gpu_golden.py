"""The sm_103a path against golden vectors produced by the reference's own GLSL
kernels: compaction, bounds, Morton keys, sort permutation, tree topology and
fill values bit-exact; bodies after each step within 1e-5 (the GPU walk uses
rsqrtf for GLSL inversesqrt, the reference restatement 1/sqrtf).  The large
fixtures (65,536 bodies) run the multi-tile sort and fill against the
reference's outputs by digest."""
import os

import pytest

from gravity_gb300 import BarnesHut

from .golden_check import fixtures, large_fixtures, replay, replay_large

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", fixtures(), ids=lambda p: os.path.basename(p))
def test_gpu_matches_reference_golden(gbh_lib, path):
    assert replay(path, BarnesHut, exact_walk=False, ordered_tasks=False)


@pytest.mark.parametrize("path", large_fixtures(), ids=lambda p: os.path.basename(p))
def test_gpu_matches_reference_large_golden(gbh_lib, path):
    assert replay_large(path, BarnesHut, exact_walk=False)
