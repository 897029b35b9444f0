"""The benchmark workloads as RadiationModel set-ups, shared by bench.py and the parity tests.

canopy_model: the plain single-band homogeneous canopy (20,000 two-sided 0.1 m leaf patches,
    LAI 2, over a one-sided 10 x 10 m ground patch; 100 direct / 300 diffuse rays, depth 3).
orchard_model: the 1 M-triangle orchard (200 trees of 5,000 3 cm leaves), bands PAR, NIR and
    longwave emission, 100 direct / 200 diffuse rays, depth 5.
Both are seeded (seed 0) synthetic scenes; ray counts can be lowered for CPU comparisons.
"""
from __future__ import annotations

import numpy as np

from . import scenes
from .radiation import Context, RadiationModel

ORCHARD_BANDS = ["LW", "NIR", "PAR"]  # std::map order, as the reference's band loop sees them


def canopy_model(n_leaves=20000, direct_rays=100, diffuse_rays=300, depth=3, device=0, mode="device"):
    sc = scenes.homogeneous_canopy(n_leaves=n_leaves, leaf=0.1, domain=10.0, zlo=1.0, zhi=3.0, seed=0)
    ctx = Context()
    ctx.addScene(sc)
    lv = sc.groups["leaves"]
    ctx.setPrimitiveData(lv, "reflectivity_SW", np.full(lv.size, 0.10))
    ctx.setPrimitiveData(lv, "transmissivity_SW", np.full(lv.size, 0.05))
    rad = RadiationModel(ctx, device=device, mode=mode)
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(30.0, 0.0))
    rad.setSourceFlux(sun, "SW", 1000.0)
    rad.setDiffuseRadiationFlux("SW", 100.0)
    rad.setDirectRayCount("SW", direct_rays)
    rad.setDiffuseRayCount("SW", diffuse_rays)
    rad.setScatteringDepth("SW", depth)
    return rad, sc


def orchard_model(leaves_per_tree=5000, nx=20, ny=10, direct_rays=100, diffuse_rays=200, depth=5, mode="device",
                  device=0):
    sc = scenes.orchard(nx=nx, ny=ny, leaves_per_tree=leaves_per_tree, side=0.03, seed=0)
    ctx = Context()
    ctx.addScene(sc)
    n = sc.n
    rng = np.random.default_rng(0)
    uu = np.arange(n)
    ctx.setPrimitiveData(uu, "reflectivity_PAR", np.full(n, 0.08))
    ctx.setPrimitiveData(uu, "transmissivity_PAR", np.full(n, 0.05))
    ctx.setPrimitiveData(uu, "reflectivity_NIR", np.full(n, 0.45))
    ctx.setPrimitiveData(uu, "transmissivity_NIR", np.full(n, 0.40))
    ctx.setPrimitiveData(uu, "emissivity_LW", np.full(n, 0.96))
    ctx.setPrimitiveData(uu, "temperature", 273.15 + rng.normal(25.0, 2.0, n))
    rad = RadiationModel(ctx, device=device, mode=mode)
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(30.0, 0.0))
    for b in ("PAR", "NIR", "LW"):
        rad.addRadiationBand(b)
        rad.setDirectRayCount(b, direct_rays)
        rad.setDiffuseRayCount(b, diffuse_rays)
        rad.setScatteringDepth(b, depth)
    rad.disableEmission("PAR")
    rad.disableEmission("NIR")
    rad.setSourceFlux(sun, "PAR", 500.0)
    rad.setSourceFlux(sun, "NIR", 450.0)
    rad.setDiffuseRadiationFlux("PAR", 50.0)
    rad.setDiffuseRadiationFlux("NIR", 45.0)
    rad.setDiffuseRadiationFlux("LW", 350.0)
    return rad, sc


def max_rel_err(got, ref, floor_frac=1e-3):
    """Largest per-primitive relative error of got against ref, with values below
    floor_frac x mean|ref| compared against that floor (near-zero fluxes)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    floor = floor_frac * max(float(np.abs(ref).mean()), 1e-30)
    return float((np.abs(got - ref) / np.maximum(np.abs(ref), floor)).max())
