"""Golden vectors (tests/golden/*.npz, written by tests/golden/make_golden.py from the
CPU FP64 oracle): the oracle must reproduce them (CPU suite), and the GPU engine must
match them -- bit for bit for the LBVH and the hits of a seeded ray set, within 1e-4
relative per primitive for fluxes, with the same ray and iteration counts."""
import os
import sys

import numpy as np
import pytest

from helios_gb300 import _hrt

from helpers import oracle_scene_for, oracle_solve

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)
import cases  # noqa: E402

FLUX_RTOL = 1e-4


def _load(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def _rel(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    floor = 1e-3 * max(float(np.abs(ref).mean()), 1e-30)
    return float((np.abs(got - ref) / np.maximum(np.abs(ref), floor)).max())


@pytest.mark.parametrize("name", sorted(cases.SOLVES))
def test_oracle_reproduces_golden(oracle_mod, name):
    g = _load(name)
    rad, labels, seed = cases.SOLVES[name]()
    flux, st = oracle_scene_for(rad, oracle_mod).run_band(oracle_solve(rad.solve_description(labels, seed=seed)))
    assert st["rays"] == int(g["rays"])
    assert st["iterations"] == int(g["iterations"])
    assert _rel(flux, g["flux"]) <= 1e-12


def test_oracle_geometry_golden(oracle_mod):
    g = _load("deep_scatter_small_geometry")
    rad, _, _ = cases.deep_scatter_small()
    sc = oracle_scene_for(rad, oracle_mod)
    codes, perm, nodes = sc.bvh()
    assert np.array_equal(codes, g["codes"]) and np.array_equal(perm, g["perm"])
    assert np.array_equal(nodes, g["nodes"])
    hit, t, face, _ = sc.trace(g["o"], g["d"])
    assert np.array_equal(hit, g["hit"])
    assert np.array_equal(t.view(np.uint32), g["t_bits"])
    assert np.array_equal(face, g["face"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.SOLVES))
def test_gpu_matches_golden(hrt_lib, name):
    g = _load(name)
    rad, labels, seed = cases.SOLVES[name]()
    rad.setSeed(seed)
    flux = rad.runBand(labels)
    assert rad.last_stats["rays"] == int(g["rays"])
    assert rad.last_stats["iterations"] == int(g["iterations"])
    worst = _rel(flux, g["flux"])
    assert worst <= FLUX_RTOL, worst


@pytest.mark.gpu
def test_gpu_geometry_golden(hrt_lib):
    g = _load("deep_scatter_small_geometry")
    rad, _, _ = cases.deep_scatter_small()
    T, ty, ts = rad.geometry_arrays()
    ctx = _hrt.Context(0)
    ctx.update_geometry(T, ty, ts, rad._bbox_faces(), rad.periodic, rad.voxel_lad())
    ctx.build_accel()
    codes, perm, nodes = ctx.bvh()
    assert np.array_equal(codes, g["codes"]) and np.array_equal(perm, g["perm"])
    assert np.array_equal(nodes[:, 12:14], g["nodes"][:, 12:14])
    assert np.array_equal(nodes[:, :12].view(np.float32), g["nodes"][:, :12].view(np.float32))
    hit, t, face = ctx.trace_rays(g["o"], g["d"])
    assert np.array_equal(hit, g["hit"])
    assert np.array_equal(t[hit >= 0].view(np.uint32), g["t_bits"][hit >= 0])
    assert np.array_equal(face, g["face"])
