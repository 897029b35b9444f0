"""The oracle's closest hits against the reference caster's stored hits
(tests/golden/reference_hits.npz, written by make_reference_hits.py from the reference's own
CollisionDetection::castRaysSoA).  Runs without the reference tree; every disagreement must
be a counted tmin / parallel / tie / grazing case (tests/refhits.py)."""
import os

import numpy as np
import pytest

import refhits

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_hits.npz")


@pytest.mark.parametrize("name", ["canopy", "orchard"])
def test_oracle_matches_reference_hits(oracle_mod, name):
    g = np.load(GOLD)
    T, ty, ts = g[f"{name}_T"], g[f"{name}_type"], g[f"{name}_twosided"]
    o, d = g[f"{name}_o"], g[f"{name}_d"]
    h, t, _, _ = oracle_mod.OracleScene(T, ty, ts).trace(o, d, mode=0)
    counts, mism = refhits.classify(T, ty, o, d, h, t, g[f"{name}_hit"], g[f"{name}_t"])
    print(name, counts)
    assert counts["mismatch"] == 0, mism[:10]
    assert counts["agree"] >= 0.999 * counts["rays"]
