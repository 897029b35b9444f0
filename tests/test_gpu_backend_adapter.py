"""GPU: the C++ drop-in adapter (helios::GB300Backend over libhrt) runs RadiationModel::runBand's
sequence of backend calls and gives the device-resident solve's fluxes.

tests/cpp/adapter_runband.cpp is compiled here with g++ and linked against libhrt.so: it fills
the reference's RayTracingGeometry / Material / Source / LaunchParams structs from a solve
description written by the Python mirror, then calls the adapter's virtuals in the order of
RadiationModel::runBand (plugins/radiation/src/RadiationModel.cpp:3779-4356, 4628-4663):
zeroRadiationBuffers, uploadSourceFluxes, launchDirectRays, getRadiationResults, the one-sided
fold, uploadRadiationOut, zeroScatterBuffers, the host emission term, launchDiffuseRays for
both faces, then per scattering iteration copyScatterToRadiation, zeroScatterBuffers,
getRadiationResults and two launchDiffuseRays.  The reference's backend interface headers are
not on a GPU machine, so the adapter compiles against tests/cpp/helios_api/RayTracingBackend.h (the
same names and types; tests/test_backend_adapter.py compiles it against the reference's own
headers where that tree is present).
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from helios_gb300 import scenes
from helios_gb300.radiation import Context, RadiationModel

from helpers import run_oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SEQ_RTOL = 1e-5   # adapter call sequence vs the device-resident solve (FP32 buffers between passes)
FLUX_RTOL = 1e-4  # vs the FP64 oracle


def _rel(got, ref):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    floor = 1e-3 * max(float(np.abs(ref).mean()), 1e-30)
    return float((np.abs(got - ref) / np.maximum(np.abs(ref), floor)).max())


@pytest.fixture(scope="module")
def driver(hrt_lib, tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("adapter") / "adapter_runband")
    build = os.path.join(ROOT, "helios_gb300", "_build")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I" + os.path.join(ROOT, "tests", "cpp", "helios_api"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "helios_gb300", "backend"),
           os.path.join(ROOT, "tests", "cpp", "adapter_runband.cpp"),
           os.path.join(ROOT, "helios_gb300", "backend", "GB300Backend.cpp"),
           "-L" + build, "-lhrt", "-Wl,-rpath," + build, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def _write_bundle(path, rad, labels, seed):
    d = rad.solve_description(labels, seed=seed)
    T, ty, ts = rad.geometry_arrays()
    bb = rad._bbox_faces()
    src = np.array([[s["type"], *s["position"], *s["width"], *s.get("rotation", (0, 0, 0))] for s in d["sources"]],
                   np.float32).reshape(-1, 9)
    arrays = {
        "T": ("f", T), "type": ("u", ty), "twosided": ("b", ts.astype(np.int8)),
        "bbox": ("f", np.zeros(0) if bb is None else np.asarray(bb)), "periodic": ("f", np.asarray(rad.periodic)),
        "rho": ("f", d["rho"]), "tau": ("f", d["tau"]), "sources": ("f", src), "source_flux": ("f", d["source_flux"]),
        "band_launch": ("b", d["band_launch"]), "depth": ("i", d["depth"]), "direct_rays": ("i", d["direct_rays"]),
        "diffuse_rays": ("i", d["diffuse_rays"]), "emission": ("b", d["emission"]), "eps": ("f", d["eps"]),
        "temperature": ("f", d["temperature"]), "diffuse_flux": ("f", d["diffuse_flux"]),
        "diffuse_ext": ("f", d["diffuse_ext"]), "diffuse_norm": ("f", d["diffuse_norm"]),
        "diffuse_peak": ("f", d["diffuse_peak"]), "prague": ("f", d["prague"]),
        "seed": ("u", np.array([d["seed"]])),
    }
    dt = {"f": np.float32, "i": np.int32, "u": np.uint32, "b": np.uint8}
    with open(path, "wb") as f:
        for name, (kind, a) in arrays.items():
            a = np.ascontiguousarray(np.asarray(a).astype(dt[kind]).reshape(-1))
            f.write(name.encode() + b"\0" + kind.encode() + struct.pack("<Q", a.size) + a.tobytes())
    return d["n"], int(d["band_launch"].sum())


def _orchard():
    sc = scenes.orchard(nx=2, ny=1, leaves_per_tree=1200, side=0.06, seed=8, ground=True)
    ctx = Context()
    ctx.addScene(sc)
    lv = sc.groups["leaves"]
    rng = np.random.default_rng(1)
    for b, r, t in (("PAR", 0.08, 0.05), ("NIR", 0.45, 0.40)):
        ctx.setPrimitiveData(lv, "reflectivity_" + b, np.full(lv.size, r))
        ctx.setPrimitiveData(lv, "transmissivity_" + b, np.full(lv.size, t))
    ctx.setPrimitiveData(lv, "emissivity_LW", np.full(lv.size, 0.96))
    ctx.setPrimitiveData(np.arange(sc.n), "temperature", 273.15 + rng.normal(25.0, 2.0, sc.n))
    rad = RadiationModel(ctx)
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(30.0, 20.0))
    for b in ("PAR", "NIR", "LW"):
        rad.addRadiationBand(b)
        rad.setDirectRayCount(b, 36)
        rad.setDiffuseRayCount(b, 64)
    rad.setScatteringDepth("PAR", 1)  # mixed depths: the launched-band compaction is exercised
    rad.setScatteringDepth("NIR", 3)
    rad.setScatteringDepth("LW", 2)
    rad.disableEmission("PAR")
    rad.disableEmission("NIR")
    rad.setSourceFlux(sun, "PAR", 500.0)
    rad.setSourceFlux(sun, "NIR", 450.0)
    rad.setDiffuseRadiationFlux("PAR", 50.0)
    rad.setDiffuseRadiationFlux("NIR", 45.0)
    rad.setDiffuseRadiationFlux("LW", 350.0)
    return rad, ["LW", "NIR", "PAR"]


def _periodic_canopy():
    sc = scenes.homogeneous_canopy(n_leaves=2000, leaf=0.1, domain=3.1623, seed=6)
    ctx = Context()
    ctx.addScene(sc)
    lv = sc.groups["leaves"]
    ctx.setPrimitiveData(lv, "reflectivity_SW", np.full(lv.size, 0.10))
    ctx.setPrimitiveData(lv, "transmissivity_SW", np.full(lv.size, 0.05))
    rad = RadiationModel(ctx)
    rad.enforcePeriodicBoundary("xy")
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(40.0, 70.0))
    rad.setSourceFlux(sun, "SW", 1000.0)
    rad.setDiffuseRadiationFlux("SW", 100.0)
    rad.setDiffuseRadiationExtinctionCoeff("SW", 0.4, scenes.sun_direction(40.0, 70.0))
    rad.setDirectRayCount("SW", 64)
    rad.setDiffuseRayCount("SW", 100)
    rad.setScatteringDepth("SW", 3)
    return rad, ["SW"]


@pytest.mark.parametrize("case", ["orchard_three_bands", "periodic_canopy_powerlaw_sky"])
def test_adapter_runband_sequence_matches_device_solve(driver, oracle_mod, tmp_path, case):
    rad, labels = _orchard() if case == "orchard_three_bands" else _periodic_canopy()
    seed = 29
    n, Bl = _write_bundle(str(tmp_path / "in.bin"), rad, labels, seed)
    r = subprocess.run([driver, str(tmp_path / "in.bin"), str(tmp_path / "flux.bin")], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "GB300" in r.stdout or "gb300" in r.stdout.lower(), r.stdout
    got = np.fromfile(str(tmp_path / "flux.bin"), np.float32).reshape(n, Bl)
    rad.setSeed(seed)
    dev = np.asarray(rad.runBand(labels), np.float64)
    assert _rel(got, dev) <= SEQ_RTOL, _rel(got, dev)
    ref, _ = run_oracle(rad, labels, oracle_mod, seed=seed)
    assert _rel(got, ref) <= FLUX_RTOL, _rel(got, ref)
