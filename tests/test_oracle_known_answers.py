"""The CPU FP64 oracle against the reference's known-answer tests
(plugins/radiation/tests/selfTest.cpp), restated as scenes + closed forms."""
import math

import numpy as np
import pytest

import scenarios
from helpers import glass_ref, run_oracle, run_oracle_cameras


@pytest.fixture(scope="module")
def run(oracle_mod):
    def _run(rad, labels, seed):
        return run_oracle(rad, labels, oracle_mod, seed=seed)[0]
    return _run


@pytest.mark.parametrize("name", ["simple_direct", "black_parallel_rectangles", "gray_parallel_rectangles",
                                  "common_edge_squares", "launch_batching", "second_law_box",
                                  "parallel_disks_masked"] + scenarios.GLASS + scenarios.SKIES)
def test_known_answer(run, name):
    res = getattr(scenarios, name)(run)
    assert not scenarios.check(res), scenarios.check(res)


def test_canopy_beer_periodic(run):
    res = scenarios.canopy_beer(run, n_leaves=6000)
    assert not scenarios.check(res), scenarios.check(res)


def test_glass_sheet_optics_reference_values(oracle_mod):
    """selfTest.cpp:9595-9615: the single-sheet model's closed-form values (n 1.5): tau(0)
    = (1 - r0) / (1 + r0) = 0.9231, no absorption when lossless, closure, the fall-off toward
    grazing incidence, and absorption for K*L = 0.05; the oracle's cosine form agrees with
    the angle form the reference's test restates."""
    tau0, rho0, a0 = glass_ref(1.0, 1.5, 0.0)
    assert abs(tau0 - 0.9231) <= 0.002 * 0.9231 and abs(a0) <= 1e-3 and abs(tau0 + rho0 + a0 - 1.0) <= 1e-4
    t60 = glass_ref(math.cos(math.radians(60)), 1.5, 0.0)[0]
    t75 = glass_ref(math.cos(math.radians(75)), 1.5, 0.0)[0]
    assert tau0 > t60 > t75 and t75 < 0.7
    ta, ra, aa = glass_ref(1.0, 1.5, 0.05)
    assert ta < tau0 and aa > 0.01 and abs(ta + ra + aa - 1.0) <= 1e-4
    c = np.cos(np.radians(np.linspace(0.0, 89.9, 400))).astype(np.float32)
    for n, kl in ((1.5, 0.0), (1.5, 0.05), (1.33, 0.2), (2.4, 1.0)):
        got = oracle_mod.glass_trs(c, n, kl)
        ref = np.array([glass_ref(float(x), n, kl) for x in c])
        assert np.abs(got - ref).max() <= 2e-5, (n, kl, np.abs(got - ref).max())


@pytest.mark.parametrize("name", scenarios.CAMERAS)
def test_camera_known_answer(oracle_mod, name):
    def run_cam(rad, labels, seed):
        return run_oracle_cameras(rad, labels, oracle_mod, seed=seed)
    res = getattr(scenarios, name)(run_cam)
    assert not scenarios.check(res, abs_tol_names=[r[0] for r in res if r[0].startswith("camera_labels")
                                                   or r[0].startswith("camera_sky_")]), scenarios.check(res)
