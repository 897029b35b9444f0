"""The CPU FP64 oracle against the reference's known-answer tests
(plugins/radiation/tests/selfTest.cpp), restated as scenes + closed forms."""
import pytest

import scenarios
from helpers import run_oracle


@pytest.fixture(scope="module")
def run(oracle_mod):
    def _run(rad, labels, seed):
        return run_oracle(rad, labels, oracle_mod, seed=seed)[0]
    return _run


@pytest.mark.parametrize("name", ["simple_direct", "black_parallel_rectangles", "gray_parallel_rectangles",
                                  "common_edge_squares", "launch_batching", "second_law_box",
                                  "parallel_disks_masked"])
def test_known_answer(run, name):
    res = getattr(scenarios, name)(run)
    assert not scenarios.check(res), scenarios.check(res)


def test_canopy_beer_periodic(run):
    res = scenarios.canopy_beer(run, n_leaves=6000)
    assert not scenarios.check(res), scenarios.check(res)
