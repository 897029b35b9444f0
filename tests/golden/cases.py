"""Small seeded radiation problems whose oracle results are frozen as golden vectors.

Each case builds a RadiationModel (helios_gb300.radiation mirror) and names the bands
it solves and the seed.  ``make_golden.py`` runs every case through the CPU FP64
oracle and writes ``<name>.npz``; ``tests/test_golden.py`` checks the oracle (CPU
suite) and the GPU engine (GPU suite) against those files.  The reference has no
per-primitive golden vectors for this path, so these pin this repository's oracle
over time and tie the GPU results to the same frozen numbers.
"""
from __future__ import annotations

import math

import numpy as np

from helios_gb300 import scenes
from helios_gb300.radiation import Context, RadiationModel


def canopy_periodic():
    sc = scenes.homogeneous_canopy(n_leaves=600, leaf=0.1, domain=math.sqrt(600 * 0.01 / 2.0), seed=3,
                                   ground_div=4)
    ctx = Context()
    ctx.addScene(sc)
    lv = sc.groups["leaves"]
    ctx.setPrimitiveData(lv, "reflectivity_SW", np.full(lv.size, 0.10))
    ctx.setPrimitiveData(lv, "transmissivity_SW", np.full(lv.size, 0.05))
    rad = RadiationModel(ctx)
    rad.enforcePeriodicBoundary("xy")
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(30.0, 0.0))
    rad.setSourceFlux(sun, "SW", 1000.0)
    rad.setDiffuseRadiationFlux("SW", 100.0)
    rad.setDirectRayCount("SW", 25)
    rad.setDiffuseRayCount("SW", 36)
    rad.setScatteringDepth("SW", 3)
    return rad, ["SW"], 11


def orchard_three_bands():
    sc = scenes.orchard(nx=1, ny=1, leaves_per_tree=600, side=0.08, seed=4, ground=True)
    ctx = Context()
    ctx.addScene(sc)
    n = sc.n
    lv = sc.groups["leaves"]
    ctx.setPrimitiveData(lv, "reflectivity_PAR", np.full(lv.size, 0.08))
    ctx.setPrimitiveData(lv, "transmissivity_PAR", np.full(lv.size, 0.05))
    ctx.setPrimitiveData(lv, "reflectivity_NIR", np.full(lv.size, 0.45))
    ctx.setPrimitiveData(lv, "transmissivity_NIR", np.full(lv.size, 0.40))
    ctx.setPrimitiveData(lv, "emissivity_LW", np.full(lv.size, 0.96))
    ctx.setPrimitiveData(np.arange(n), "temperature", 273.15 + 25.0 + 2.0 * np.sin(np.arange(n)))
    rad = RadiationModel(ctx)
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(40.0, 60.0))
    for b in ("PAR", "NIR", "LW"):
        rad.addRadiationBand(b)
        rad.setDirectRayCount(b, 16)
        rad.setDiffuseRayCount(b, 25)
        rad.setScatteringDepth(b, 2)
    rad.disableEmission("PAR")
    rad.disableEmission("NIR")
    rad.setSourceFlux(sun, "PAR", 500.0)
    rad.setSourceFlux(sun, "NIR", 450.0)
    rad.setDiffuseRadiationFlux("PAR", 50.0)
    rad.setDiffuseRadiationFlux("NIR", 45.0)
    rad.setDiffuseRadiationFlux("LW", 350.0)
    return rad, ["LW", "NIR", "PAR"], 5


def sources_all_types():
    sc = scenes.homogeneous_canopy(n_leaves=300, leaf=0.15, domain=2.0, seed=6)
    ctx = Context()
    ctx.addScene(sc)
    rad = RadiationModel(ctx)
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    rad.setDirectRayCount("SW", 16)
    rad.setScatteringDepth("SW", 0)
    s = [rad.addCollimatedRadiationSource(scenes.sun_direction(20.0, 10.0)),
         rad.addSphereRadiationSource((1.0, 1.0, 6.0), 0.5),
         rad.addSunSphereRadiationSource(scenes.sun_direction(50.0, 200.0)),
         rad.addRectangleRadiationSource((0.5, 1.5, 5.0), (1.0, 2.0), (0.1, 0.2, 0.0)),
         rad.addDiskRadiationSource((1.5, 0.5, 4.0), 0.7, (0.0, 0.3, 0.5))]
    for k, src in enumerate(s):
        rad.setSourceFlux(src, "SW", 100.0 * (k + 1))
    return rad, ["SW"], 9


def deep_scatter_small():
    sc = scenes.deep_scatter(n_tri=1200, n_patch=200, n_disk=200, vox_div=3, domain=2.0, height=1.0, seed=7)
    ctx = Context()
    ctx.addScene(sc)
    n = sc.n
    ctx.setPrimitiveData(np.arange(1, n), "reflectivity_NIR", np.full(n - 1, 0.45))
    ctx.setPrimitiveData(np.arange(1, n), "transmissivity_NIR", np.full(n - 1, 0.40))
    rad = RadiationModel(ctx)
    rad.enforcePeriodicBoundary("xy")
    rad.addRadiationBand("NIR")
    rad.disableEmission("NIR")
    rad.setDirectRayCount("NIR", 9)
    rad.setDiffuseRayCount("NIR", 16)
    rad.setDiffuseRadiationFlux("NIR", 100.0)
    rad.setScatteringDepth("NIR", 20)
    rad.setScatteringResidualTolerance(1e-4)
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(25.0, 45.0))
    rad.setSourceFlux(sun, "NIR", 400.0)
    return rad, ["NIR"], 3


SOLVES = {"canopy_periodic": canopy_periodic, "orchard_three_bands": orchard_three_bands,
          "sources_all_types": sources_all_types, "deep_scatter_small": deep_scatter_small}


def ray_set(seed=12, n=4000):
    """Seeded explicit rays through the deep_scatter_small box, for hit-ID vectors."""
    rng = np.random.default_rng(seed)
    o = np.stack([rng.uniform(-0.2, 2.2, n), rng.uniform(-0.2, 2.2, n), rng.uniform(-0.5, 1.5, n)], 1)
    return o.astype(np.float32), scenes.uniform_sphere(rng, n).astype(np.float32)
