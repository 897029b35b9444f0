"""GPU: passes split into primitive chunks give the solve of one launch, and the device
error word reaches the caller without a fault.

Ray ids inside a trace launch are 32-bit; passes of 2^31 rays or more are planned on the
host as consecutive launches over primitive chunks.  These tests never run such a size:
they lower the per-launch limit (hrt_set_launch_ray_limit) so a small scene goes through
many chunks, and compare with the same solve in one launch and with the FP64 oracle.
"""
import math

import numpy as np
import pytest

from helios_gb300 import _hrt, scenes
from helios_gb300.radiation import Context, RadiationModel

from helpers import run_oracle

pytestmark = pytest.mark.gpu

FLUX_RTOL = 1e-4  # per-primitive relative flux error vs the FP64 oracle
CHUNK_RTOL = 1e-6  # chunked vs one launch: only the order of FP64 sums differs, then FP32 rounding


def _rel_err(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    floor = 1e-3 * max(float(np.abs(ref).mean()), 1e-30)
    return float((np.abs(got - ref) / np.maximum(np.abs(ref), floor)).max())


def _canopy(mode="device", n_leaves=2000, depth=2, periodic=True):
    sc = scenes.homogeneous_canopy(n_leaves=n_leaves, leaf=0.1, domain=math.sqrt(n_leaves * 0.01 / 2.0), seed=4)
    ctx = Context()
    ctx.addScene(sc)
    ctx.setPrimitiveData(sc.groups["leaves"], "reflectivity_SW", np.full(n_leaves, 0.10))
    ctx.setPrimitiveData(sc.groups["leaves"], "transmissivity_SW", np.full(n_leaves, 0.05))
    rad = RadiationModel(ctx, mode=mode)
    if periodic:
        rad.enforcePeriodicBoundary("xy")
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(35, 20))
    rad.setSourceFlux(sun, "SW", 1000.0)
    rad.setDiffuseRadiationFlux("SW", 100.0)
    rad.setDirectRayCount("SW", 100)
    rad.setDiffuseRayCount("SW", 100)
    rad.setScatteringDepth("SW", depth)
    rad.setSeed(31)
    return rad


@pytest.mark.parametrize("mode", ["device", "backend"])
def test_chunked_passes_equal_one_launch(oracle_mod, mode):
    rad = _canopy(mode=mode)
    one = rad.runBand("SW").astype(np.float64)
    k_one = rad.last_stats.get("kernels")
    # 30,000 rays per launch: direct passes (100 rays) in chunks of 300 primitives, diffuse
    # passes (100 rays x 2 faces) in chunks of 150: 7 and 14 launches per pass
    rad.ctx.set_launch_ray_limit(30_000)
    try:
        many = rad.runBand("SW").astype(np.float64)
        k_many = rad.last_stats.get("kernels")
    finally:
        rad.ctx.set_launch_ray_limit(1 << 31)
    assert _rel_err(many, one) <= CHUNK_RTOL
    ref, st = run_oracle(rad, ["SW"], oracle_mod, seed=31)
    assert _rel_err(many, ref) <= FLUX_RTOL
    if mode == "device":
        assert rad.last_stats["rays"] == st["rays"]
        assert k_many > k_one  # the passes really ran as several launches
    assert rad.ctx.device_status() == 0


def test_chunked_sweep_equals_one_launch():
    sc = scenes.orchard(nx=2, ny=1, leaves_per_tree=700, side=0.06, seed=5, ground=True)
    n = sc.n
    rho = np.full((n, 2), 0.3, np.float32)
    tau = np.full((n, 2), 0.2, np.float32)
    g = _hrt.Context(0)
    g.update_geometry(sc.T, sc.ptype, sc.twosided)
    g.build_accel()
    dirs, direct, diffuse, _ = scenes.day_sweep(n=4)
    a = g.run_sweep(dirs, direct, diffuse, rho, tau, 36, 49, 2, seed=9).astype(np.float64)
    g.set_launch_ray_limit(20_000)  # recording launches of 49 rays x 2 faces: 204 primitives each
    try:
        b = g.run_sweep(dirs, direct, diffuse, rho, tau, 36, 49, 2, seed=9).astype(np.float64)
    finally:
        g.set_launch_ray_limit(1 << 31)
    assert _rel_err(b, a) <= CHUNK_RTOL
    assert g.device_status() == 0


def test_visit_budget_exhaustion_is_reported_and_cleared():
    """A node-visit budget of 2 ends every ray's traversal early: the solve returns
    HRT_EDEVICE with the budget named, the word is cleared, and the next solve with the
    default budget is clean and equals a solve that never saw the error."""
    rad = _canopy(n_leaves=800, depth=1)
    before = rad.runBand("SW").astype(np.float64)
    rad.ctx.set_visit_budget(2)
    try:
        with pytest.raises(_hrt.HrtError) as e:
            rad.runBand("SW")
    finally:
        rad.ctx.set_visit_budget(0)
    assert e.value.code == _hrt.HRT_EDEVICE
    assert "visit budget" in str(e.value)
    assert rad.ctx.device_status() == 0  # the failing call cleared the word
    after = rad.runBand("SW").astype(np.float64)
    assert rad.ctx.device_status() == 0
    assert _rel_err(after, before) <= CHUNK_RTOL
