"""The CPU oracle against golden vectors produced by the reference's own GLSL
kernels (tests/golden, generated by tests/golden/make_golden.py): every stage
output and the bodies after each step must be bit-identical."""
import os

import pytest

from .golden_check import fixtures, large_fixtures, replay, replay_large


@pytest.mark.parametrize("path", fixtures(), ids=lambda p: os.path.basename(p))
def test_oracle_matches_reference_golden(oracle_mod, path):
    assert replay(path, oracle_mod.OracleBarnesHut, exact_walk=True, ordered_tasks=True)


@pytest.mark.parametrize("path", large_fixtures(), ids=lambda p: os.path.basename(p))
def test_oracle_matches_reference_large_golden(oracle_mod, path):
    assert replay_large(path, oracle_mod.OracleBarnesHut, exact_walk=True)


def test_golden_fixtures_present():
    assert len(fixtures()) >= 4
    assert len(large_fixtures()) >= 2
