"""GPU closest hits against hits computed by the REFERENCE's own CPU ray caster.

tests/golden/reference_hits.npz holds, for two seeded scenes, 8,000 free-space rays and the
hit index and distance that CollisionDetection::castRaysSoA (plugins/collisiondetection/src/
CollisionDetection_RayTracing.cpp:551-680), compiled from the reference tree, returned
(make_reference_hits.py).  The device traversal must agree except for counted tmin /
parallel / tie / grazing cases (tests/refhits.py), and must equal the oracle bit for bit.
"""
import os

import numpy as np
import pytest

from helios_gb300 import _hrt

import refhits

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_hits.npz")


@pytest.mark.parametrize("name", ["canopy", "orchard"])
def test_device_hits_match_reference_caster(hrt_lib, oracle_mod, name):
    g = np.load(GOLD)
    T, ty, ts = g[f"{name}_T"], g[f"{name}_type"], g[f"{name}_twosided"]
    o, d = g[f"{name}_o"], g[f"{name}_d"]
    ctx = _hrt.Context(0)
    ctx.update_geometry(T, ty, ts)
    ctx.build_accel()
    hit, t, _ = ctx.trace_rays(o, d)
    counts, mism = refhits.classify(T, ty, o, d, hit, t, g[f"{name}_hit"], g[f"{name}_t"])
    print(name, counts)
    assert counts["mismatch"] == 0, mism[:10]
    assert counts["agree"] >= 0.999 * counts["rays"]
    h2, t2, _, _ = oracle_mod.OracleScene(T, ty, ts).trace(o, d, mode=0)
    assert np.array_equal(hit, h2)
    assert np.array_equal(t[hit >= 0], t2[h2 >= 0])
    assert ctx.device_status() == 0
