"""The oracle's closest hits against the REFERENCE's own CPU ray caster (CPU only).

The reference's CollisionDetection plug-in (castRaysSoA, plugins/collisiondetection/src/
CollisionDetection_RayTracing.cpp:551-680) is compiled from the reference tree by
oracle/ref.mk and given the same FP32 transforms.  It has its own BVH and its own triangle
and patch tests; the oracle (and the GPU, which matches the oracle bit for bit) uses a
watertight test over an LBVH.  On seeded free-space rays every hit-ID disagreement must be
a counted tmin, parallel, tie or grazing case (tests/refhits.py); real mismatches must be zero.
Skips where the reference tree is absent (the GPU machine).
"""
import math

import numpy as np
import pytest

from helios_gb300 import scenes

import refhits

refcast = pytest.importorskip("refcast")
if not refcast.available():
    pytest.skip("reference tree not present", allow_module_level=True)

NRAYS = 200_000
MAX_COUNTED = 1e-3  # counted (tmin + parallel + tie + grazing) disagreements per ray, at most


def _compare(oracle_mod, T, ty, ts, lo, hi, seed):
    ref = refcast.RefScene(T, ty)
    o, d = refhits.free_space_rays(lo, hi, NRAYS, seed)
    ri, rt = ref.cast(o, d)
    h, t, _, _ = oracle_mod.OracleScene(T, ty, ts).trace(o, d, mode=0)
    counts, mism = refhits.classify(T, ty, o, d, h, t, ri, rt)
    print(counts)
    assert counts["mismatch"] == 0, mism[:10]
    counted = counts["tmin"] + counts["parallel"] + counts["tie"] + counts["grazing"]
    assert counted <= MAX_COUNTED * NRAYS, counts
    both = (h >= 0) & (ri >= 0) & (h == ri)
    assert both.sum() > 0.2 * NRAYS
    # the distances of agreeing hits differ only by the rounding of two different FP32 tests,
    # which grows as 1/cos toward grazing incidence
    rel = np.abs(t[both].astype(np.float64) - rt[both]) / np.maximum(rt[both], 1e-3)
    assert np.percentile(rel, 99.9) < 1e-4 and rel.max() < 1e-2, (np.percentile(rel, 99.9), rel.max())
    return counts


def test_canopy_patches_vs_reference_caster(oracle_mod):
    sc = scenes.homogeneous_canopy(n_leaves=20000, leaf=0.1, domain=10.0, seed=0)
    _compare(oracle_mod, sc.T, sc.ptype, sc.twosided, (-1, -1, 0), (11, 11, 4), seed=11)


def test_orchard_triangles_vs_reference_caster(oracle_mod):
    sc = scenes.orchard(nx=4, ny=2, leaves_per_tree=5000, side=0.03, seed=0, ground=True)
    _compare(oracle_mod, sc.T, sc.ptype, sc.twosided, (-2, -2, 0), (17, 7, 5.5), seed=12)


def test_dense_crown_grazing_is_counted(oracle_mod):
    """Large triangles packed into one crown: many edge-adjacent hits, all classified."""
    sc = scenes.orchard(nx=1, ny=1, leaves_per_tree=20000, side=0.12, radii=(0.8, 0.8, 1.0), seed=4)
    _compare(oracle_mod, sc.T, sc.ptype, sc.twosided, (-1.5, -1.5, 1.5), (1.5, 1.5, 4.5), seed=13)


def test_reference_caster_sees_our_transforms(oracle_mod):
    """Rays aimed at each primitive's centre hit that primitive in both tracers."""
    sc = scenes.homogeneous_canopy(n_leaves=2000, leaf=0.1, domain=math.sqrt(2000 * 0.01 / 2.0), seed=3)
    T = sc.T.reshape(-1, 4, 4).astype(np.float64)
    centre = T[:, :3, 3]
    nrm = np.cross(T[:, :3, 0], T[:, :3, 1])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    o = (centre + 0.05 * nrm).astype(np.float32)
    d = (-nrm).astype(np.float32)
    ri, _ = refcast.RefScene(sc.T, sc.ptype).cast(o, d)
    h, _, _, _ = oracle_mod.OracleScene(sc.T, sc.ptype, sc.twosided).trace(o, d, mode=0)
    assert np.array_equal(ri, h)
    assert (h == np.arange(sc.n)).mean() > 0.9  # most centres are not hidden by a nearer leaf
