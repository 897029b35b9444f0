"""Regenerate reference_hits.npz: closest hits computed by the REFERENCE's own CPU ray caster.

    python tests/golden/make_reference_hits.py     (needs the reference tree; see oracle/refcast.py)

For two small scenes -- a 2,000-leaf patch canopy over a ground patch and a 3,000-triangle
orchard crown pair over a ground patch -- stores the transforms, types and two-sided flags,
8,000 seeded free-space rays each, and the hit index (-1 = miss) and distance that
CollisionDetection::castRaysSoA (plugins/collisiondetection/src/
CollisionDetection_RayTracing.cpp:551-680), compiled from the reference tree by
oracle/ref.mk, returns for them.  The GPU test (tests/test_gpu_reference_hits.py) compares
device hits with these on a box that has no reference tree.
"""
from __future__ import annotations

import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import numpy as np  # noqa: E402

import refcast  # noqa: E402
import refhits  # noqa: E402
from helios_gb300 import scenes  # noqa: E402

NRAYS = 8000


def cases():
    dom = math.sqrt(2000 * 0.01 / 2.0)
    c = scenes.homogeneous_canopy(n_leaves=2000, leaf=0.1, domain=dom, seed=21)
    yield "canopy", c, (-0.5, -0.5, 0.0), (dom + 0.5, dom + 0.5, 3.5), 31
    o = scenes.orchard(nx=2, ny=1, leaves_per_tree=1500, side=0.06, radii=(0.9, 0.9, 1.2), seed=22, ground=True)
    yield "orchard", o, (-1.5, -1.5, 0.0), (6.5, 1.5, 4.5), 32


def main():
    out = {}
    for name, sc, lo, hi, seed in cases():
        o, d = refhits.free_space_rays(lo, hi, NRAYS, seed)
        idx, t = refcast.RefScene(sc.T, sc.ptype).cast(o, d)
        out.update({f"{name}_T": sc.T.astype(np.float32), f"{name}_type": sc.ptype.astype(np.uint32),
                    f"{name}_twosided": sc.twosided.astype(np.int8), f"{name}_o": o, f"{name}_d": d,
                    f"{name}_hit": idx.astype(np.int32), f"{name}_t": t.astype(np.float32)})
        print(name, sc.n, "primitives,", int((idx >= 0).sum()), "of", NRAYS, "rays hit")
    np.savez_compressed(os.path.join(HERE, "reference_hits.npz"), **out)


if __name__ == "__main__":
    main()
