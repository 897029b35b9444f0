"""Cameras on the GPU: the reference's camera tests, pixels / labels / depths against the
FP64 oracle, the granular backend calls against the device-resident solve, and tiling."""
import math

import numpy as np
import pytest

from helios_gb300 import scenes
from helios_gb300.radiation import Context, RadiationModel

import scenarios
from helpers import run_device_cameras, run_oracle_cameras

pytestmark = pytest.mark.gpu

PIX_RTOL = 1e-4  # relative pixel error vs the FP64 oracle (floor 1e-3 of the image mean)


@pytest.mark.parametrize("name", scenarios.CAMERAS)
def test_camera_known_answers_on_gpu(name):
    res = getattr(scenarios, name)(run_device_cameras)
    abs_names = [r[0] for r in res if r[0].startswith("camera_labels") or r[0].startswith("camera_sky_")]
    assert not scenarios.check(res, abs_tol_names=abs_names), scenarios.check(res)


def _canopy_with_cameras(periodic=False, mode="device", seed=0):
    """Leaves over a ground with a sun and a sky in two bands; a pinhole camera looking down
    and an oblique camera with a lens and 9 samples per pixel."""
    sc = scenes.homogeneous_canopy(n_leaves=2000, leaf=0.1, domain=3.0, zlo=0.5, zhi=2.0, seed=seed)
    ctx = Context()
    ctx.addScene(sc)
    lv = sc.groups["leaves"]
    ctx.setPrimitiveData(lv, "reflectivity_SW", np.full(lv.size, 0.10))
    ctx.setPrimitiveData(lv, "transmissivity_SW", np.full(lv.size, 0.05))
    ctx.setPrimitiveData(lv, "reflectivity_NIR", np.full(lv.size, 0.45))
    ctx.setPrimitiveData(lv, "transmissivity_NIR", np.full(lv.size, 0.40))
    rad = RadiationModel(ctx, mode=mode)
    if periodic:
        rad.enforcePeriodicBoundary("xy")
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(30, 40))
    for b, f in (("SW", 800.0), ("NIR", 600.0)):
        rad.addRadiationBand(b)
        rad.disableEmission(b)
        rad.setSourceFlux(sun, b, f)
        rad.setDiffuseRadiationFlux(b, 100.0)
        rad.setDirectRayCount(b, 36)
        rad.setDiffuseRayCount(b, 64)
        rad.setScatteringDepth(b, 2)
    rad.setCameraSkyRadiance("SW", 30.0)
    rad.addRadiationCamera("top", ["SW", "NIR"], (1.5, 1.5, 6.0), (1.5, 1.5, 0.0),
                           {"camera_resolution": (48, 40), "HFOV": 40.0, "lens_diameter": 0.0}, 1)
    rad.addRadiationCamera("side", ["SW"], (0.3, 0.2, 2.8), (2.0, 2.5, 0.8),
                           {"camera_resolution": (40, 32), "HFOV": 60.0, "lens_diameter": 0.05,
                            "focal_plane_distance": 3.0}, 9)
    return rad


def _pix_close(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    floor = 1e-3 * max(float(np.abs(ref).mean()), 1e-30)
    return float((np.abs(got - ref) / np.maximum(np.abs(ref), floor)).max())


@pytest.mark.parametrize("periodic", [False, True])
def test_cameras_vs_oracle(oracle_mod, periodic):
    """Pixels within 1e-4 of the oracle; pixel labels and depths bit-exact (the same FP32 rays
    and hits)."""
    rad = _canopy_with_cameras(periodic=periodic)
    f1, c1 = run_device_cameras(rad, ["SW", "NIR"], 17)
    f2, c2 = run_oracle_cameras(rad, ["SW", "NIR"], oracle_mod, seed=17)
    assert set(c1) == set(c2) == {"top", "side"}
    for k in c1:
        assert np.array_equal(c1[k]["labels"], c2[k]["labels"]), k
        assert np.array_equal(c1[k]["depths"], c2[k]["depths"]), k
        err = _pix_close(c1[k]["pixels"], c2[k]["pixels"])
        assert err <= PIX_RTOL, (k, err)
        assert float(c1[k]["pixels"].max()) > 0.0
    frac_sky = float(np.mean(c1["side"]["labels"] == 0))
    assert 0.0 < frac_sky < 1.0


def test_camera_backend_calls_match_device_solve():
    """launchCameraRays / launchPixelLabelRays / getCameraResults through the backend entry
    points, with the camera view accumulated on the host, give the device-resident images."""
    a = _canopy_with_cameras(mode="device")
    b = _canopy_with_cameras(mode="backend")
    _, ca = run_device_cameras(a, ["SW", "NIR"], 5)
    _, cb = run_device_cameras(b, ["SW", "NIR"], 5)
    for k in ca:
        assert np.array_equal(ca[k]["labels"], cb[k]["labels"])
        assert np.array_equal(ca[k]["depths"], cb[k]["depths"])
        assert _pix_close(cb[k]["pixels"], ca[k]["pixels"]) <= 1e-5


def test_camera_tiles_match_one_launch():
    """Tiles of a camera (the reference's tiled launches) accumulate the image of one launch:
    rays are keyed by global pixel, not by tile."""
    rad = _canopy_with_cameras()
    rad.setSeed(3)
    rad.runBand(["SW", "NIR"])
    desc = rad.solve_description(["SW", "NIR"], seed=3)
    cam = dict(desc["cameras"][1])
    ctx = rad.ctx
    W, H = cam["resolution"]
    other = dict(cam, camera_id=99, resolution=(4, 4), antialiasing=1)
    ctx.launch_camera(other)  # a launch of another camera: the next launch of cam starts a fresh image
    ctx.launch_camera(cam)
    full = ctx.get_camera_results(W, H, 2, labels=False)[0]
    ctx.launch_camera(other)
    for oy, th in ((0, 13), (13, H - 13)):
        for ox, tw in ((0, 25), (25, W - 25)):
            t = dict(cam, tile_offset=(ox, oy), tile_resolution=(tw, th))
            ctx.launch_camera(t)
    tiled = ctx.get_camera_results(W, H, 2, labels=False)[0]
    assert _pix_close(tiled, full) <= 1e-6
    ctx.zero_camera_pixel_buffers(W, H)
    for ox, tw in ((0, 7), (7, W - 7)):
        ctx.launch_pixel_labels(dict(cam, tile_offset=(ox, 0), tile_resolution=(tw, H)))
    _, lab, dep = ctx.get_camera_results(W, H, 2, pixels=False)
    ctx.zero_camera_pixel_buffers(W, H)
    ctx.launch_pixel_labels(cam)
    _, lab1, dep1 = ctx.get_camera_results(W, H, 2, pixels=False)
    assert np.array_equal(lab, lab1) and np.array_equal(dep, dep1)


def test_camera_errors():
    rad = _canopy_with_cameras()
    rad.setSeed(1)
    rad.runBand(["SW", "NIR"])
    desc = rad.solve_description(["SW", "NIR"], seed=1)
    cam = dict(desc["cameras"][0])
    with pytest.raises(RuntimeError, match="tile"):
        rad.ctx.launch_camera(dict(cam, tile_offset=(40, 0), tile_resolution=(20, 10)))
    with pytest.raises(RuntimeError, match="antialiasing"):
        rad.ctx.launch_camera(dict(cam, antialiasing=0))
    with pytest.raises(RuntimeError, match="resolution"):
        rad.ctx.get_camera_results(7, 7, 2)
    with pytest.raises(Exception, match="antialiasing"):
        rad.addRadiationCamera("bad", ["SW"], (0, 0, 1), (0, 0, 0), None, 0)
