"""The sm_103a path against golden vectors produced by the reference's own GLSL
kernels: compaction, bounds, Morton keys, sort permutation, tree topology and
fill values bit-exact; bodies after each step within 1e-5 (the GPU walk uses
rsqrtf for GLSL inversesqrt, the reference restatement 1/sqrtf)."""
import os

import pytest

from gravity_gb300 import BarnesHut

from .golden_check import fixtures, replay

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", fixtures(), ids=lambda p: os.path.basename(p))
def test_gpu_matches_reference_golden(gbh_lib, path):
    assert replay(path, BarnesHut, exact_walk=False, ordered_tasks=False)
