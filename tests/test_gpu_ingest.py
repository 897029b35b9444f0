"""Geometry read from files into the solve and the served stream: a PLY orchard tree solved
against the oracle, and an OBJ canopy registered with the server."""
import struct

import numpy as np
import pytest

from helios_gb300 import _hrt, scenes
from helios_gb300.radiation import Context, RadiationModel

from helpers import run_oracle

pytestmark = pytest.mark.gpu


def _tree_vertices(leaves=3000, seed=2):
    sc = scenes.orchard(nx=1, ny=1, leaves_per_tree=leaves, side=0.05, seed=seed, ground=False)
    T = sc.T.astype(np.float64).reshape(-1, 4, 4)
    v0 = T[:, :3, 3]
    v1 = v0 + T[:, :3, 1]
    v2 = v1 + T[:, :3, 0]
    return np.stack([v0, v1, v2], axis=1).astype(np.float32)


def _write_ply(path, V):
    n = V.shape[0]
    head = ["ply", "format binary_little_endian 1.0", f"element vertex {3 * n}", "property float x",
            "property float y", "property float z", f"element face {n}", "property list uchar int vertex_indices",
            "end_header"]
    data = V.reshape(-1, 3).astype("<f4").tobytes()
    data += b"".join(struct.pack("<Biii", 3, 3 * k, 3 * k + 1, 3 * k + 2) for k in range(n))
    path.write_bytes(("\n".join(head) + "\n").encode() + data)
    return str(path)


def test_ply_tree_solve_vs_oracle(oracle_mod, tmp_path):
    V = _tree_vertices()
    ctx = Context()
    ctx.addPatch((0.0, 0.0, 0.0), (8.0, 8.0))
    ctx.setPrimitiveData(0, "twosided_flag", 0)
    u = ctx.loadPLY(_write_ply(tmp_path / "tree.ply", V), origin=(0.0, 0.0, 0.5), upaxis="ZUP")
    assert len(u) == V.shape[0]
    ctx.setPrimitiveData(u, "reflectivity_SW", np.full(len(u), 0.1))
    ctx.setPrimitiveData(u, "transmissivity_SW", np.full(len(u), 0.05))
    rad = RadiationModel(ctx)
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(40, 30))
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    rad.setSourceFlux(sun, "SW", 900.0)
    rad.setDiffuseRadiationFlux("SW", 120.0)
    rad.setDirectRayCount("SW", 49)
    rad.setDiffuseRayCount("SW", 100)
    rad.setScatteringDepth("SW", 3)
    rad.setSeed(11)
    got = rad.runBand("SW")
    ref, st = run_oracle(rad, ["SW"], oracle_mod, seed=11)
    floor = 1e-3 * float(np.abs(ref).mean())
    err = np.abs(got - ref) / np.maximum(np.abs(ref), floor)
    assert err.max() <= 1e-4, err.max()
    assert rad.last_stats["rays"] == st["rays"]


def test_obj_canopy_served(tmp_path, hrt_lib):
    """An OBJ canopy (quad leaves) registered with the server gives the same fluxes as the
    same arrays solved alone."""
    rng = np.random.default_rng(5)
    lines = []
    for k in range(2000):
        c = rng.uniform((0.0, 0.0, 0.5), (4.0, 4.0, 2.5))
        e1, e2 = rng.normal(size=3) * 0.06, rng.normal(size=3) * 0.06
        for q in (c, c + e1, c + e1 + e2, c + e2):
            lines.append("v %.6f %.6f %.6f" % tuple(q))
        b = 4 * k + 1
        lines.append(f"f {b} {b + 1} {b + 2} {b + 3}")
    p = tmp_path / "canopy.obj"
    p.write_text("\n".join(lines) + "\n")
    f = _hrt.load_scene_file(str(p))
    n = f["T"].shape[0]
    assert n == 4000
    rho, tau = np.full((n, 1), 0.1), np.full((n, 1), 0.05)
    srv = _hrt.Server(device=0, workers=2, hbm_budget=1 << 30)
    srv.add_scene(0, f["T"], f["type"], f["twosided"], rho, tau)
    bands = np.array([1], np.uint8)
    sun = scenes.sun_direction(30, 0)
    srv.submit(1, 0, 0.0, bands, sun, np.array([800.0]), np.array([100.0]), 36, 64, 2, 7, keep=True)
    srv.start()
    srv.wait()
    res = srv.result(1, n)
    alone = _hrt.Context(0)
    alone.update_geometry(f["T"], f["type"], f["twosided"])
    alone.build_accel()
    desc = {"band_launch": bands, "sources": [{"type": 0, "position": tuple(sun)}], "source_flux": np.array([800.0]),
            "rho": rho, "tau": tau, "diffuse_flux": np.array([100.0]), "direct_rays": np.array([36]),
            "diffuse_rays": np.array([64]), "depth": np.array([2]), "emission": np.zeros(1, np.uint8), "seed": 7}
    ref = alone.run_band(desc).reshape(-1)
    floor = 1e-3 * float(np.abs(ref).mean())
    err = np.abs(res["flux"].astype(np.float64) - ref) / np.maximum(np.abs(ref), floor)
    assert err.max() <= 1e-5, err.max()
    srv.close()
