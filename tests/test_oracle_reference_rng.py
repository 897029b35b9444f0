"""Statistical parity with the reference's Monte-Carlo estimator.

The reference draws every ray from a TEA-16 seeded 24-bit LCG stream with a wall-clock
launch seed (OptiX8DeviceCode.cu:29-49, :1232, :1497; RadiationModel.cpp:3961), so its
results can be matched only in distribution.  The oracle's reference-RNG mode draws from
that stream; K seeded solves with it and K seeded Philox solves (the stream the device
reproduces bit for bit) agree per primitive within 3 standard errors for >= 99 % of the
primitives that carry flux, and in the area-weighted canopy totals.
"""
import math

import numpy as np
import pytest

from helios_gb300 import scenes
from helios_gb300.radiation import Context, RadiationModel

from helpers import ensemble, oracle_scene_for, run_oracle, z_scores

K = 24


def canopy(n_leaves=800, depth=3, periodic=True, ndiff=144):
    """Homogeneous canopy (spherical leaf angles, LAI 2) over a one-sided ground: sun at 30 deg
    and an isotropic sky, rho 0.10 / tau 0.05, 100 direct and ndiff diffuse rays, depth 3."""
    sc = scenes.homogeneous_canopy(n_leaves=n_leaves, leaf=0.1, domain=math.sqrt(n_leaves * 0.01 / 2.0), seed=3,
                                   ground_div=4)
    ctx = Context()
    ctx.addScene(sc)
    ctx.setPrimitiveData(sc.groups["leaves"], "reflectivity_SW", np.full(n_leaves, 0.10))
    ctx.setPrimitiveData(sc.groups["leaves"], "transmissivity_SW", np.full(n_leaves, 0.05))
    rad = RadiationModel(ctx)
    if periodic:
        rad.enforcePeriodicBoundary("xy")
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(30, 0))
    rad.setSourceFlux(sun, "SW", 1000.0)
    rad.setDiffuseRadiationFlux("SW", 100.0)
    rad.setDirectRayCount("SW", 100)
    rad.setDiffuseRayCount("SW", ndiff)
    rad.setScatteringDepth("SW", depth)
    return rad, sc


def check_statistical_parity(a, b, area):
    z = z_scores(a, b)
    assert z.size > 100
    assert (np.abs(z) <= 3.0).mean() >= 0.99, np.sort(np.abs(z))[-10:]
    ta, tb = a @ area, b @ area
    zt = (ta.mean() - tb.mean()) / math.sqrt(ta.var(ddof=1) / len(ta) + tb.var(ddof=1) / len(tb))
    assert abs(zt) <= 3.0, zt


def test_reference_stream_differs_from_philox(oracle_mod):
    """The reference-RNG mode really draws another ray set (same seed, other fluxes)."""
    rad, _ = canopy(n_leaves=300, depth=1)
    scene = oracle_scene_for(rad, oracle_mod)
    a, _ = run_oracle(rad, ["SW"], oracle_mod, scene=scene, seed=5)
    with oracle_mod.reference_rng():
        b, _ = run_oracle(rad, ["SW"], oracle_mod, scene=scene, seed=5)
    c, _ = run_oracle(rad, ["SW"], oracle_mod, scene=scene, seed=5)
    assert not np.array_equal(a, b)
    assert np.array_equal(a, c)  # the mode is restored on exit


def test_philox_estimator_matches_reference_estimator(oracle_mod):
    rad, sc = canopy()
    scene = oracle_scene_for(rad, oracle_mod)
    seeds = range(100, 100 + K)
    philox = ensemble(lambda s: run_oracle(rad, ["SW"], oracle_mod, scene=scene, seed=s)[0], seeds)
    with oracle_mod.reference_rng():
        ref = ensemble(lambda s: run_oracle(rad, ["SW"], oracle_mod, scene=scene, seed=s + 1000)[0], seeds)
    check_statistical_parity(philox, ref, sc.area)
