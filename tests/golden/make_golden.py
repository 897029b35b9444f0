"""Regenerate the golden vectors in this directory from the CPU FP64 oracle.

    python tests/golden/make_golden.py

Writes, per solve case of cases.py, ``<case>.npz`` with the per-primitive flux
[n, bands] (float64), the traced-ray count and the scattering iterations run; and
``deep_scatter_small_geometry.npz`` with the host LBVH (Morton codes, permutation,
nodes) and the closest hits (primitive, distance bits, face) of a seeded ray set.
Run it only when the oracle's arithmetic changes on purpose, and say why in the commit.
"""
from __future__ import annotations

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests"), HERE):
    sys.path.insert(0, p)

import numpy as np  # noqa: E402

import cases  # noqa: E402
import oracle  # noqa: E402
from helpers import oracle_scene_for, oracle_solve  # noqa: E402


def main():
    oracle.build()
    for name, make in cases.SOLVES.items():
        rad, labels, seed = make()
        sc = oracle_scene_for(rad, oracle)
        flux, st = sc.run_band(oracle_solve(rad.solve_description(labels, seed=seed)), threads=1)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), flux=flux, rays=st["rays"],
                            iterations=st["iterations"], labels=np.array(labels))
        print(name, flux.shape, st["rays"], st["iterations"])
    rad, _, _ = cases.deep_scatter_small()
    sc = oracle_scene_for(rad, oracle)
    codes, perm, nodes = sc.bvh()
    o, d = cases.ray_set()
    hit, t, face, _ = sc.trace(o, d)
    np.savez_compressed(os.path.join(HERE, "deep_scatter_small_geometry.npz"), codes=codes, perm=perm, nodes=nodes,
                        o=o, d=d, hit=hit, t_bits=t.view(np.uint32), face=face)
    print("geometry", codes.shape, (hit >= 0).mean())


if __name__ == "__main__":
    main()
