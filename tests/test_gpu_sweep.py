"""Batched day sweep (hrt_run_sweep): every channel equals the plain runBand it stands for."""
import numpy as np
import pytest

from helios_gb300 import scenes
from helios_gb300.radiation import Context, RadiationModel

pytestmark = pytest.mark.gpu


def _orchard(mode="device"):
    sc = scenes.orchard(nx=2, ny=2, leaves_per_tree=800, side=0.06, seed=3, ground=True)
    ctx = Context()
    ctx.addScene(sc)
    lv = sc.groups["leaves"]
    ctx.setPrimitiveData(lv, "reflectivity_PAR", np.full(lv.size, 0.08))
    ctx.setPrimitiveData(lv, "transmissivity_PAR", np.full(lv.size, 0.05))
    ctx.setPrimitiveData(lv, "reflectivity_NIR", np.full(lv.size, 0.45))
    ctx.setPrimitiveData(lv, "transmissivity_NIR", np.full(lv.size, 0.40))
    rad = RadiationModel(ctx, mode=mode)
    for b in ("PAR", "NIR"):
        rad.addRadiationBand(b)
        rad.disableEmission(b)
        rad.setDirectRayCount(b, 49)
        rad.setDiffuseRayCount(b, 64)
        rad.setScatteringDepth(b, 3)
    return rad, sc


def test_sweep_channels_equal_plain_solves():
    rad, sc = _orchard()
    dirs, direct, diffuse, _ = scenes.day_sweep(n=8)
    # force one twilight channel (sky only) to exercise the sequence without a direct pass
    direct[2, :] = 0.0
    diffuse[2, :] = [20.0, 15.0]
    rad.updateGeometry()
    desc = rad.solve_description(["PAR", "NIR"])
    n = sc.n
    rho = desc["rho"][0]  # [n, Bg] (bands in std::map order: NIR, PAR)
    tau = desc["tau"][0]
    order = ["NIR", "PAR"]
    sweep = rad.ctx.run_sweep(dirs, direct[:, ::-1], diffuse[:, ::-1], rho, tau, 49, 64, 3, seed=123)
    assert sweep.shape == (n, 8, 2)
    sun = 0  # the collimated source solve_description() created (Philox source slot 0)
    assert len(rad.sources) == 1
    for s in range(8):
        for bi, band in enumerate(order):
            rad.sources[sun]["position"] = tuple(float(x) for x in dirs[s])
            rad.setSourceFlux(sun, band, float(direct[s, 1 - bi]))
            rad.setDiffuseRadiationFlux(band, float(diffuse[s, 1 - bi]))
            rad.setSeed(123)
            plain = rad.runBand(band)[:, 0].astype(np.float64)
            got = sweep[:, s, bi].astype(np.float64)
            floor = 1e-3 * max(float(np.abs(plain).mean()), 1e-30)
            err = np.abs(got - plain) / np.maximum(np.abs(plain), floor)
            assert err.max() <= 1e-5, (s, band, err.max())
    # a replay of the captured graph gives the same numbers
    again = rad.ctx.run_sweep(dirs, direct[:, ::-1], diffuse[:, ::-1], rho, tau, 49, 64, 3, seed=123)
    np.testing.assert_allclose(again, sweep, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("variant", [4, 6, 7, 8, 9, 10, 11, 12, 13])
def test_sweep_recording_variants_agree(variant):
    """The recording trace of the sweep gives the same channels whichever 4-wide kernel
    records the hits (the generic persistent kernel or the lean one in each of its block
    shapes and shared stack depths)."""
    rad, sc = _orchard()
    dirs, direct, diffuse, _ = scenes.day_sweep(n=4)
    rad.updateGeometry()
    desc = rad.solve_description(["PAR", "NIR"])
    rho, tau = desc["rho"][0], desc["tau"][0]
    base = rad.ctx.run_sweep(dirs, direct, diffuse, rho, tau, 49, 64, 2, seed=7).astype(np.float64)
    rad.ctx.set_tuning(16 + variant)
    try:
        got = rad.ctx.run_sweep(dirs, direct, diffuse, rho, tau, 49, 64, 2, seed=7).astype(np.float64)
    finally:
        rad.ctx.set_tuning(1)
    np.testing.assert_allclose(got, base, rtol=1e-6, atol=1e-9)
    assert rad.ctx.device_status() == 0


def _scene_ctx(kind):
    from helios_gb300 import _hrt

    if kind == "orchard":
        sc = scenes.orchard(nx=2, ny=2, leaves_per_tree=600, side=0.06, seed=11, ground=True)
        bbox, per = None, (0.0, 0.0)
    elif kind == "periodic":
        sc = scenes.homogeneous_canopy(n_leaves=1500, leaf=0.1, domain=2.7386, seed=12)
        ctx = Context()
        ctx.addScene(sc)
        rad = RadiationModel(ctx)
        rad.enforcePeriodicBoundary("xy")
        bbox, per = rad._bbox_faces(), rad.periodic  # the mirror's periodic walls
    else:
        sc = scenes.homogeneous_canopy(n_leaves=300, leaf=0.2, domain=2.0, seed=13)
        bbox, per = None, (0.0, 0.0)
    c = _hrt.Context(0)
    c.update_geometry(sc.T, sc.ptype, sc.twosided, bbox, per)
    c.build_accel()
    return c, sc


def test_multi_scene_sweep_equals_each_scene_alone():
    """Three scenes of different sizes, suns, bands, ray counts and depths (one with periodic
    walls) in one multi-scene graph: every pass of all scenes is one persistent launch, and each
    scene's channels and ray count equal its own sweep's."""
    specs = []
    for kind, nsun, nb, dr, fr, depth, seed in (("orchard", 4, 2, 36, 49, 3, 5), ("periodic", 3, 1, 16, 64, 2, 6),
                                                 ("small", 2, 3, 25, 36, 0, 7)):
        c, sc = _scene_ctx(kind)
        dirs, direct, diffuse, _ = scenes.day_sweep(n=nsun)
        direct = np.repeat(direct[:, :1], nb, axis=1) * np.linspace(1.0, 0.6, nb)
        diffuse = np.repeat(diffuse[:, :1], nb, axis=1) * np.linspace(1.0, 0.8, nb)
        rng = np.random.default_rng(seed)
        rho = rng.uniform(0.05, 0.45, (sc.n, nb)).astype(np.float32)
        tau = (0.8 * rng.uniform(0.0, 1.0, (sc.n, nb)) * (1 - rho)).astype(np.float32)
        specs.append((c, dict(sun_dir=dirs, direct_flux=direct, diffuse_flux=diffuse, rho=rho, tau=tau,
                              direct_rays=dr, diffuse_rays=fr, depth=depth, seed=seed)))
    alone, rays = [], []
    for c, sw in specs:
        alone.append(c.run_sweep(**sw).astype(np.float64))
        rays.append(c.last_stats()["rays"])
    from helios_gb300 import _hrt

    for _ in range(2):  # capture, then replay
        multi = _hrt.run_sweep_multi([c for c, _ in specs], [sw for _, sw in specs])
        for k, (c, _) in enumerate(specs):
            np.testing.assert_allclose(multi[k], alone[k], rtol=1e-6, atol=1e-9)
            assert c.last_stats()["rays"] == rays[k]
            assert c.device_status() == 0
