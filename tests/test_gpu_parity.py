"""GPU parity: libhrt (sm_103a) against the CPU oracle through the C ABI.

Bit-exact: device LBVH vs host build, generated ray sets, hit IDs / distances /
faces.  Flux: per-primitive relative error <= 1e-4 against the FP64 oracle on
the same seeded ray set (FP32 geometry, FP64 accumulation on both sides).
"""
import math

import numpy as np
import pytest

from helios_gb300 import _hrt, scenes
from helios_gb300.radiation import Context, RadiationModel

import scenarios
from helpers import ensemble, oracle_solve, oracle_scene_for, run_oracle

pytestmark = pytest.mark.gpu

FLUX_RTOL = 1e-4  # spec tolerance: per-primitive relative flux error vs the FP64 oracle


def _mixed(seed=1, n_leaf=3000, n_tri=3000, leaf=0.3):
    a = scenes.homogeneous_canopy(n_leaves=n_leaf, leaf=leaf, domain=5, seed=seed)
    b = scenes.orchard(nx=1, ny=1, leaves_per_tree=n_tri, side=leaf, seed=seed + 1)
    return (np.concatenate([a.T, b.T]), np.concatenate([a.ptype, b.ptype]), np.concatenate([a.twosided, b.twosided]))


@pytest.fixture(scope="module")
def gpu(hrt_lib):
    return _hrt.Context(0)


def _flux_close(got, ref, rtol=FLUX_RTOL):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    floor = 1e-3 * max(float(np.abs(ref).mean()), 1e-30)
    err = np.abs(got - ref) / np.maximum(np.abs(ref), floor)
    return float(err.max()), err


@pytest.mark.parametrize("n", [1, 2, 3, 17, 4096, 6000])
def test_bvh_bit_exact(gpu, oracle_mod, n):
    T, ty, ts = _mixed(seed=n)
    T, ty, ts = T[:n], ty[:n], ts[:n]
    gpu.update_geometry(T, ty, ts)
    gpu.build_accel()
    c1, p1, n1 = gpu.bvh()
    c2, p2, n2 = oracle_mod.OracleScene(T, ty, ts).bvh()
    assert np.array_equal(c1, c2)
    assert np.array_equal(p1, p2)
    assert np.array_equal(n1[:, 12:14], n2[:, 12:14])
    assert np.array_equal(n1[:, :12].view(np.float32), n2[:, :12].view(np.float32))


@pytest.mark.parametrize("kind,face", [(0, 1), (1, 1), (1, 0)])
def test_ray_sets_bit_exact(gpu, oracle_mod, kind, face):
    T, ty, ts = _mixed(seed=4, n_leaf=500, n_tri=500)
    gpu.update_geometry(T, ty, ts)
    gpu.build_accel()
    sc = oracle_mod.OracleScene(T, ty, ts)
    sun = scenes.sun_direction(30, 0)
    o1, d1 = gpu.gen_rays(kind, 1234, 7, 100 if kind == 0 else 324, face, sun)
    o2, d2 = sc.gen_rays(kind, 1234, 7, 100 if kind == 0 else 324, face, sun)
    assert np.array_equal(o1, o2)
    assert np.array_equal(d1, d2)


@pytest.mark.parametrize("anyhit", [False, True])
def test_hit_ids_exact(gpu, oracle_mod, anyhit):
    T, ty, ts = _mixed(seed=9)
    gpu.update_geometry(T, ty, ts)
    gpu.build_accel()
    sc = oracle_mod.OracleScene(T, ty, ts)
    rng = np.random.default_rng(2)
    n = 200000
    o = np.stack([rng.uniform(-1, 6, n), rng.uniform(-1, 6, n), rng.uniform(0, 6, n)], 1).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    h1, t1, f1 = gpu.trace_rays(o, d, anyhit=anyhit)
    h2, t2, f2, _ = sc.trace(o, d, mode=3 if anyhit else 0)
    if anyhit:
        assert np.array_equal(h1 >= 0, h2 >= 0)
    else:
        assert np.array_equal(h1, h2)
        assert np.array_equal(t1[h1 >= 0], t2[h2 >= 0])
        assert np.array_equal(f1, f2)
    assert gpu.device_status() == 0


def _canopy_model(n_leaves=2000, depth=3, periodic=False, mode="device", ground_div=1):
    sc = scenes.homogeneous_canopy(n_leaves=n_leaves, leaf=0.1, domain=math.sqrt(n_leaves * 0.01 / 2.0), seed=0,
                                   ground_div=ground_div)
    ctx = Context()
    ctx.addScene(sc)
    ctx.setPrimitiveData(sc.groups["leaves"], "reflectivity_SW", np.full(n_leaves, 0.10))
    ctx.setPrimitiveData(sc.groups["leaves"], "transmissivity_SW", np.full(n_leaves, 0.05))
    rad = RadiationModel(ctx, mode=mode)
    if periodic:
        rad.enforcePeriodicBoundary("xy")
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(30, 0))
    rad.setSourceFlux(sun, "SW", 1000.0)
    rad.setDiffuseRadiationFlux("SW", 100.0)
    rad.setDirectRayCount("SW", 100)
    rad.setDiffuseRayCount("SW", 300)
    rad.setScatteringDepth("SW", depth)
    return rad


@pytest.mark.parametrize("periodic", [False, True])
def test_canopy_flux_vs_oracle(oracle_mod, periodic):
    rad = _canopy_model(periodic=periodic)
    rad.setSeed(77)
    got = rad.runBand("SW")
    ref, st = run_oracle(rad, ["SW"], oracle_mod, seed=77)
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst
    assert rad.last_stats["rays"] == st["rays"]


def test_many_onesided_before_twosided(oracle_mod):
    """A 40 x 40 one-sided ground tile comes first, so the bottom-face ray range starts with
    1600 x 324 rays that the face rule skips; every later two-sided primitive must still be traced."""
    rad = _canopy_model(n_leaves=1500, depth=1, periodic=True, ground_div=40)
    rad.setSeed(17)
    got = rad.runBand("SW")
    ref, st = run_oracle(rad, ["SW"], oracle_mod, seed=17)
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst
    assert rad.last_stats["rays"] == st["rays"]


def test_backend_sequence_matches_device_solve(oracle_mod):
    a = _canopy_model(mode="device")
    b = _canopy_model(mode="backend")
    a.setSeed(5)
    b.setSeed(5)
    fa = a.runBand("SW")
    fb = b.runBand("SW")
    worst, _ = _flux_close(fb, fa, 1e-5)
    assert worst <= 1e-5, worst


def _orchard_model(trees=(2, 1), leaves=1500, mode="device"):
    sc = scenes.orchard(nx=trees[0], ny=trees[1], leaves_per_tree=leaves, side=0.05, seed=0, ground=True)
    ctx = Context()
    ctx.addScene(sc)
    n = sc.n
    lv = sc.groups["leaves"]
    rng = np.random.default_rng(0)
    ctx.setPrimitiveData(lv, "reflectivity_PAR", np.full(lv.size, 0.08))
    ctx.setPrimitiveData(lv, "transmissivity_PAR", np.full(lv.size, 0.05))
    ctx.setPrimitiveData(lv, "reflectivity_NIR", np.full(lv.size, 0.45))
    ctx.setPrimitiveData(lv, "transmissivity_NIR", np.full(lv.size, 0.40))
    ctx.setPrimitiveData(lv, "emissivity_LW", np.full(lv.size, 0.96))
    ctx.setPrimitiveData(np.arange(n), "temperature", 273.15 + rng.normal(25.0, 2.0, n))
    rad = RadiationModel(ctx, mode=mode)
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(30, 0))
    for b in ("PAR", "NIR", "LW"):
        rad.addRadiationBand(b)
        rad.setDirectRayCount(b, 100)
        rad.setDiffuseRayCount(b, 200)
        rad.setScatteringDepth(b, 5)
    for b in ("PAR", "NIR"):
        rad.disableEmission(b)
        rad.setDiffuseRadiationFlux(b, 100.0)
    rad.setSourceFlux(sun, "PAR", 500.0)
    rad.setSourceFlux(sun, "NIR", 450.0)
    return rad


def test_orchard_three_bands_vs_oracle(oracle_mod):
    rad = _orchard_model()
    rad.setSeed(3)
    got = rad.runBand(["PAR", "NIR", "LW"])
    ref, st = run_oracle(rad, ["PAR", "NIR", "LW"], oracle_mod, seed=3)
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst


def test_orchard_backend_sequence(oracle_mod):
    a, b = _orchard_model(), _orchard_model(mode="backend")
    a.setSeed(8)
    b.setSeed(8)
    fa = a.runBand(["PAR", "NIR", "LW"])
    fb = b.runBand(["PAR", "NIR", "LW"])
    worst, _ = _flux_close(fb, fa, 1e-5)
    assert worst <= 1e-5, worst


def test_mixed_depth_band_compaction(oracle_mod):
    """Bands with different scattering depths run together: the launched-band
    compaction of the reference's scattering loop (RadiationModel.cpp:4250-4276)."""
    rad = _orchard_model(leaves=800)
    rad.setScatteringDepth("PAR", 1)
    rad.setScatteringDepth("NIR", 3)
    rad.setScatteringDepth("LW", 2)
    rad.setSeed(13)
    got = rad.runBand(["PAR", "NIR", "LW"])
    ref, _ = run_oracle(rad, ["PAR", "NIR", "LW"], oracle_mod, seed=13)
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst


def test_sources_all_types(oracle_mod):
    """Sphere, sun-sphere, rectangle and disk sources (OptiX8DeviceCode.cu:1341-1415)."""
    ctx = Context()
    ctx.addScene(scenes.homogeneous_canopy(n_leaves=400, leaf=0.2, domain=3, seed=2))
    rad = RadiationModel(ctx)
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    s = [rad.addSphereRadiationSource((1.0, 1.0, 6.0), 0.5),
         rad.addSunSphereRadiationSource(scenes.sun_direction(40, 30)),
         rad.addRectangleRadiationSource((2.0, 1.0, 5.0), (1.0, 2.0), (0.1, 0.2, 0.3)),
         rad.addDiskRadiationSource((0.5, 2.0, 5.5), 0.7, (0.0, 0.3, 0.0))]
    for k, f in zip(s, (300.0, 800.0, 150.0, 120.0)):
        rad.setSourceFlux(k, "SW", f)
    rad.setDirectRayCount("SW", 64)
    rad.setScatteringDepth("SW", 0)
    rad.setSeed(21)
    got = rad.runBand("SW")
    desc = rad.solve_description(["SW"])
    sc = oracle_scene_for(rad, oracle_mod)
    ref, _ = sc.run_band(oracle_solve(desc, rotation=_hrt.source_rotation))
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst


@pytest.mark.parametrize("name", ["simple_direct", "black_parallel_rectangles", "gray_parallel_rectangles",
                                  "common_edge_squares", "launch_batching", "second_law_box",
                                  "parallel_disks_masked"] + scenarios.GLASS + scenarios.SKIES)
def test_known_answers_on_gpu(name):
    def run(rad, labels, seed):
        rad.setSeed(seed)
        return rad.runBand(labels)
    res = getattr(scenarios, name)(run)
    assert not scenarios.check(res), scenarios.check(res)


@pytest.mark.parametrize("sky", ["powerlaw", "prague"])
def test_anisotropic_sky_canopy_vs_oracle(oracle_mod, sky):
    """Sun + anisotropic sky over a periodic canopy with scattering: the sky factor of every
    escaping diffuse ray (OptiX8DeviceCode.cu:148-164, power-law psi^-K normalised over the
    hemisphere, or the Prague pattern with its zenith normalisation) matches the FP64 oracle
    per primitive within 1e-4 on the same ray set."""
    rad = _canopy_model(n_leaves=2500, depth=2, periodic=True)
    if sky == "powerlaw":
        rad.setDiffuseRadiationExtinctionCoeff("SW", 0.6, scenes.sun_direction(35, 120))
    else:
        ctx = rad.context
        ctx.setGlobalData("sky_spectrum", [(400.0, 1.0), (550.0, 1.0), (700.0, 1.0)])
        rad.setDiffuseSpectrum("sky_spectrum")
        ctx.setGlobalData("prague_sky_valid", 1)
        ctx.setGlobalData("prague_sky_sun_direction", tuple(scenes.sun_direction(30, 0)))
        ctx.setGlobalData("prague_sky_spectral_params", [450.0, 0.12, 6.0, 12.0, 1.8, 0.0,
                                                          650.0, 0.08, 3.0, 20.0, 1.4, 0.0])
    rad.setSeed(37)
    got = rad.runBand("SW")
    desc = rad.solve_description(["SW"])
    if sky == "prague":
        assert desc["prague"][0, 3] > 0 and desc["diffuse_ext"][0] == 0
    else:
        assert desc["diffuse_ext"][0] > 0
    ref, st = run_oracle(rad, ["SW"], oracle_mod, seed=37)
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst
    assert rad.last_stats["rays"] == st["rays"]
    # the anisotropic sky changes the answer (the test is not passing on an isotropic sky)
    iso = _canopy_model(n_leaves=2500, depth=2, periodic=True)
    iso.setSeed(37)
    assert np.abs(np.asarray(iso.runBand("SW"), np.float64) - got).max() > 1e-3 * np.abs(got).max()


def test_spectral_materials_per_source_vs_oracle(oracle_mod):
    """Leaves whose reflectivity and transmissivity are spectra (global data named by primitive
    data), two suns with different spectra: each source sees its own band-averaged materials
    ([source][primitive][band], RadiationModel.cpp:2400-2470), which the direct pass reads per
    source and the diffuse passes from source 0 (OptiX8DeviceCode.cu:1612).  GPU vs the FP64
    oracle within 1e-4 per primitive, over two bands."""
    rad = _canopy_model(n_leaves=2000, depth=2, periodic=True)
    ctx = rad.context
    lv = np.arange(1, ctx.getPrimitiveCount())
    ctx.setGlobalData("leaf_rho", [(400, 0.05), (500, 0.10), (600, 0.08), (700, 0.45), (800, 0.50), (900, 0.48)])
    ctx.setGlobalData("leaf_tau", [(400, 0.02), (500, 0.05), (600, 0.04), (700, 0.40), (800, 0.45), (900, 0.44)])
    ctx.setGlobalData("sun_a", [(400, 1.5), (500, 2.0), (600, 1.8), (700, 1.2), (800, 1.0), (900, 0.8)])
    ctx.setGlobalData("sun_b", [(400, 0.2), (600, 1.0), (900, 2.0)])
    ctx.setPrimitiveData(lv, "reflectivity_spectrum", "leaf_rho")
    ctx.setPrimitiveData(lv, "transmissivity_spectrum", "leaf_tau")
    for b in ("reflectivity_SW", "transmissivity_SW"):  # leave the band constants at their defaults
        ctx.primitive_data.pop(b, None)
        ctx.bulk_data.pop(b, None)
    rad.bands.pop("SW")
    for b, lo, hi in (("VIS", 400, 700), ("NIR", 700, 900)):
        rad.addRadiationBand(b, lo, hi)
        rad.disableEmission(b)
        rad.setDirectRayCount(b, 64)
        rad.setDiffuseRayCount(b, 100)
        rad.setScatteringDepth(b, 2)
        rad.setDiffuseRadiationFlux(b, 60.0)
    rad.sources.clear()
    a = rad.addCollimatedRadiationSource(scenes.sun_direction(30, 0))
    c = rad.addCollimatedRadiationSource(scenes.sun_direction(55, 140))
    rad.setSourceSpectrum(a, "sun_a")
    rad.setSourceSpectrum(c, "sun_b")
    for b, fa, fc in (("VIS", 500.0, 200.0), ("NIR", 450.0, 300.0)):
        rad.setSourceFlux(a, b, fa)
        rad.setSourceFlux(c, b, fc)
    desc = rad.solve_description(["NIR", "VIS"])
    assert not np.allclose(desc["rho"][0], desc["rho"][1])  # the sources see different materials
    rad.setSeed(41)
    got = rad.runBand(["NIR", "VIS"])
    ref, st = run_oracle(rad, ["NIR", "VIS"], oracle_mod, seed=41)
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst
    assert rad.last_stats["rays"] == st["rays"]


def test_canopy_beer_reference_size():
    """The reference's periodic canopy test at its own size: 20 x 20 m, LAI 2, 5 cm
    leaves (160,000 patches), 1000 direct / 5000 diffuse rays (selfTest.cpp:1625-1717)."""
    def run(rad, labels, seed):
        rad.setSeed(seed)
        return rad.runBand(labels)
    res = scenarios.canopy_beer(run, n_leaves=160000, leaf=0.05, ndir=1000, ndiff=5000, ground_div=100)
    assert not scenarios.check(res), scenarios.check(res)


def test_errors_and_edge_cases(gpu):
    with pytest.raises(_hrt.HrtError):
        gpu.update_geometry(np.zeros((1, 16), np.float32), [7], [1])  # unsupported primitive type
    g2 = _hrt.Context(0)
    with pytest.raises(_hrt.HrtError):
        g2.trace_rays(np.zeros((1, 3)), np.ones((1, 3)))  # no acceleration structure yet
    g2.update_geometry(np.zeros((0, 16), np.float32), np.zeros(0), np.zeros(0))
    g2.build_accel()
    h, t, f = g2.trace_rays(np.zeros((4, 3)), np.ones((4, 3)))
    assert (h == -1).all()
    # a zero diffuse ray count is a no-op launch (OptiX8Backend.cpp:968-970)
    ctx = Context()
    ctx.addPatch((0, 0, 0), (1, 1))
    rad = RadiationModel(ctx)
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    rad.setDiffuseRadiationFlux("SW", 10.0)
    rad.setDiffuseRayCount("SW", 0)
    f = rad.runBand("SW")
    assert f.shape == (1, 1) and f[0, 0] == 0.0


def test_determinism_and_energy_bound():
    """Same seed, same flux.  With periodic walls a canopy lit by the sun alone (or the
    sky alone) absorbs at most what enters its top."""
    rad = _canopy_model(n_leaves=4000, depth=3, periodic=True)
    rad.setSeed(99)
    f1 = rad.runBand("SW").astype(np.float64)
    rad.setSeed(99)
    f2 = rad.runBand("SW").astype(np.float64)
    np.testing.assert_allclose(f1, f2, rtol=1e-6, atol=1e-6)
    T, ty, area = rad.context.arrays()
    (x0, x1), (y0, y1), _ = rad.context.getDomainBoundingBox()
    top = (x1 - x0) * (y1 - y0)
    rad.setDiffuseRadiationFlux("SW", 0.0)
    sun = float((rad.runBand("SW")[:, 0] * area).sum())
    assert sun <= 1000.0 * math.cos(math.radians(30)) * top * 1.005
    rad.setDiffuseRadiationFlux("SW", 100.0)
    rad.setSourceFlux(0, "SW", 0.0)
    sky = float((rad.runBand("SW")[:, 0] * area).sum())
    assert sky <= 100.0 * top * 1.01


def test_sun_plus_sky_nonadditivity_matches_reference(oracle_mod):
    """RadiationModel::runBand with direct + diffuse + scattering and no emission gathers the
    direct-scattered energy twice and drops the sky's first scatter (RadiationModel.cpp:4236-4298),
    so runBand(sun+sky) != runBand(sun) + runBand(sky).  The drop-in reproduces that sequence."""
    def total(sun, sky, engine):
        rad = _canopy_model(n_leaves=1500, depth=3, periodic=True)
        rad.setSourceFlux(0, "SW", sun)
        rad.setDiffuseRadiationFlux("SW", sky)
        rad.setSeed(31)
        if engine == "gpu":
            f = rad.runBand("SW")
        else:
            f, _ = run_oracle(rad, ["SW"], oracle_mod, seed=31)
        return float((np.asarray(f)[:, 0] * rad.context.arrays()[2]).sum())
    g = [total(1000, 0, "gpu"), total(0, 100, "gpu"), total(1000, 100, "gpu")]
    o = [total(1000, 0, "cpu"), total(0, 100, "cpu"), total(1000, 100, "cpu")]
    np.testing.assert_allclose(g, o, rtol=1e-6)
    excess = g[2] - g[0] - g[1]
    assert excess > 0.01 * g[2]


def test_traversal_counts_match_oracle(gpu, oracle_mod):
    """The statistics kernels count the same node visits as the host traversal of the same
    binary BVH (measure flag 4 selects the binary tree for the counting launches)."""
    rad = _canopy_model(n_leaves=1500, depth=0)
    rad.setSeed(4)
    rad.ctx.set_measure(1 | 4)
    rad.runBand("SW")
    m = rad.ctx.get_measure()
    rad.ctx.set_measure(0)
    _, st = run_oracle(rad, ["SW"], oracle_mod, seed=4)
    assert m["node_visits"] == st["nodes"]
    assert m["prim_tests"] == st["prims"]
    # the diffuse launches' share of the counts (the bench's roofline reads it)
    assert 0 < m["diffuse_node_visits"] < m["node_visits"]
    assert 0 < m["diffuse_prim_tests"] <= m["prim_tests"]


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13])
def test_traversal_variants_agree(oracle_mod, variant):
    """Every diffuse-kernel variant (binary or compressed 4-wide nodes, persistent or one
    ray per thread) gives the oracle's fluxes and ray count: hits do not depend on the
    tree's width or the visiting order (closest hit, ties to the smaller index)."""
    rad = _canopy_model(n_leaves=2500, depth=2, periodic=True)
    rad.ctx.set_tuning(16 + variant)
    rad.setSeed(31)
    got = rad.runBand("SW")
    rad.ctx.set_tuning(1)
    ref, st = run_oracle(rad, ["SW"], oracle_mod, seed=31)
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst
    assert rad.last_stats["rays"] == st["rays"]
    assert rad.ctx.device_status() == 0


def test_ray_budget_keeps_results(oracle_mod):
    """With a per-thread ray budget the persistent trace retires blocks early and launches
    more of them; every ray is still traced once, so fluxes and ray counts stay the same."""
    rad = _canopy_model(n_leaves=2500, depth=2, periodic=True)
    rad.setSeed(33)
    base = rad.runBand("SW")
    rays = rad.last_stats["rays"]
    for budget in (1, 7, 32):
        rad.ctx.set_ray_budget(budget)
        rad.setSeed(33)
        got = rad.runBand("SW")
        worst, _ = _flux_close(got, base, 1e-6)
        assert worst <= 1e-6, (budget, worst)
        assert rad.last_stats["rays"] == rays
    rad.ctx.set_ray_budget(0)
    assert rad.ctx.device_status() == 0


def _masked_canopy(n_leaves=1500, seed=3):
    """Canopy of square leaves masked to disks (every second one with texture coordinates
    that show only a quarter of the mask) and triangles masked to half, over a ground."""
    rng = np.random.default_rng(seed)
    ctx = Context()
    ctx.addPatch((1.5, 1.5, 0.0), (3.0, 3.0))
    ctx.setPrimitiveData(0, "twosided_flag", 0)
    m = scenarios.disk_mask(64)
    half = np.zeros((32, 32), np.uint8)
    half[:, :16] = 1
    for k in range(n_leaves):
        c = rng.uniform((0.2, 0.2, 0.3), (2.8, 2.8, 2.5))
        rot = (rng.uniform(0.0, 0.5 * math.pi), rng.uniform(0.0, 2.0 * math.pi))
        uv = [(0.5, 0.5), (1.0, 0.5), (1.0, 1.0), (0.5, 1.0)] if k % 2 else None
        ctx.addPatch(tuple(c), (0.2, 0.2), rot, texture_mask=m, uv=uv)
    for k in range(n_leaves // 2):
        p0 = rng.uniform((0.2, 0.2, 0.5), (2.8, 2.8, 2.5))
        e1, e2 = rng.normal(size=3) * 0.1, rng.normal(size=3) * 0.1
        uv = [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0)] if k % 3 == 0 else None
        ctx.addTriangle(tuple(p0), tuple(p0 + e1), tuple(p0 + e2), texture_mask=half, uv=uv)
    n = ctx.getPrimitiveCount()
    ctx.setPrimitiveData(np.arange(1, n), "reflectivity_SW", np.full(n - 1, 0.2))
    ctx.setPrimitiveData(np.arange(1, n), "transmissivity_SW", np.full(n - 1, 0.1))
    rad = RadiationModel(ctx)
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(35, 10))
    rad.setSourceFlux(sun, "SW", 800.0)
    rad.setDiffuseRadiationFlux("SW", 100.0)
    rad.setDirectRayCount("SW", 36)
    rad.setDiffuseRayCount("SW", 64)
    rad.setScatteringDepth("SW", 2)
    return rad, ctx


def test_masked_canopy_vs_oracle(oracle_mod):
    """Texture-masked patches (with and without texture coordinates) and triangles: the
    oracle's fluxes and ray counts."""
    rad, _ = _masked_canopy()
    rad.setSeed(9)
    got = rad.runBand("SW")
    ref, st = run_oracle(rad, ["SW"], oracle_mod, seed=9)
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst
    assert rad.last_stats["rays"] == st["rays"]


def test_masked_hits_and_rays_exact(oracle_mod):
    """Hits through masked primitives and the ray sets of masked origins are bit-exact."""
    rad, ctx = _masked_canopy(n_leaves=600, seed=4)
    rad.updateGeometry()
    sc = oracle_scene_for(rad, oracle_mod)
    rng = np.random.default_rng(6)
    n = 100000
    o = np.stack([rng.uniform(-0.5, 3.5, n), rng.uniform(-0.5, 3.5, n), rng.uniform(0.0, 3.0, n)], 1)
    d = scenes.uniform_sphere(rng, n)
    h1, t1, f1 = rad.ctx.trace_rays(o.astype(np.float32), d.astype(np.float32))
    h2, t2, f2, _ = sc.trace(o, d)
    assert np.array_equal(h1, h2) and np.array_equal(t1[h1 >= 0], t2[h2 >= 0]) and np.array_equal(f1, f2)
    for kind, face in ((0, 0), (1, 1), (1, 0)):
        o1, d1 = rad.ctx.gen_rays(kind, 5, 2, 64, face, scenes.sun_direction(35, 10))
        o2, d2 = sc.gen_rays(kind, 5, 2, 64, face, scenes.sun_direction(35, 10))
        assert np.array_equal(o1, o2) and np.array_equal(d1, d2)


def _greenhouse(periodic=False, mode="device", n_leaves=1500, seed=0):
    """A canopy under a roof of 16 slightly tilted glass panes (glass in PAR and NIR with
    absorption, opaque in LW), two suns and a sky; leaves and ground emit in LW."""
    sc = scenes.homogeneous_canopy(n_leaves=n_leaves, leaf=0.1, domain=3.0, zlo=0.5, zhi=2.0, seed=seed)
    ctx = Context()
    ctx.addScene(sc)
    lv = sc.groups["leaves"]
    roof = [ctx.addPatch((0.375 + 0.75 * i, 0.375 + 0.75 * j, 2.6 + 0.05 * ((i + j) % 2)), (0.75, 0.75),
                         (0.08 * (i - 1.5), 0.3 * j)) for i in range(4) for j in range(4)]
    ctx.setPrimitiveData(lv, "reflectivity_PAR", np.full(lv.size, 0.08))
    ctx.setPrimitiveData(lv, "transmissivity_PAR", np.full(lv.size, 0.05))
    ctx.setPrimitiveData(lv, "reflectivity_NIR", np.full(lv.size, 0.45))
    ctx.setPrimitiveData(lv, "transmissivity_NIR", np.full(lv.size, 0.40))
    ctx.setPrimitiveData(lv, "emissivity_LW", np.full(lv.size, 0.96))
    for k, u in enumerate(roof):
        ctx.setPrimitiveData(u, "glass_n_PAR", 1.5)
        ctx.setPrimitiveData(u, "glass_KL_PAR", 0.05)
        ctx.setPrimitiveData(u, "glass_n_NIR", 1.45 + 0.01 * k)
        ctx.setPrimitiveData(u, "glass_KL_NIR", 0.2)
        ctx.setPrimitiveData(u, "emissivity_LW", 0.9)
    n = ctx.getPrimitiveCount()
    rng = np.random.default_rng(seed)
    ctx.setPrimitiveData(np.arange(n), "temperature", 273.15 + rng.normal(25.0, 2.0, n))
    rad = RadiationModel(ctx, mode=mode)
    if periodic:
        rad.enforcePeriodicBoundary("xy")
    s0 = rad.addCollimatedRadiationSource(scenes.sun_direction(35, 20))
    s1 = rad.addCollimatedRadiationSource(scenes.sun_direction(60, 200))
    for b in ("PAR", "NIR", "LW"):
        rad.addRadiationBand(b)
        rad.setDirectRayCount(b, 64)
        rad.setDiffuseRayCount(b, 100)
        rad.setScatteringDepth(b, 3)
    for b, f0, f1 in (("PAR", 500.0, 120.0), ("NIR", 450.0, 90.0)):
        rad.disableEmission(b)
        rad.setDiffuseRadiationFlux(b, 100.0)
        rad.setSourceFlux(s0, b, f0)
        rad.setSourceFlux(s1, b, f1)
    return rad


@pytest.mark.parametrize("periodic", [False, True])
def test_greenhouse_glass_vs_oracle(oracle_mod, periodic):
    """Translucent covers: two suns and the sky through a glass roof (glass in every launched
    band of the PAR + NIR launch), then LW with the roof opaque; fluxes of every primitive,
    covers included, and the ray count against the oracle."""
    rad = _greenhouse(periodic=periodic)
    rad.setSeed(13)
    got = rad.runBand(["PAR", "NIR"])
    ref, st = run_oracle(rad, ["PAR", "NIR"], oracle_mod, seed=13)
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst
    assert rad.last_stats["rays"] == st["rays"]
    rad.setSeed(14)
    got = rad.runBand("LW")
    ref, _ = run_oracle(rad, ["LW"], oracle_mod, seed=14)
    worst, _ = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst


def test_greenhouse_backend_sequence():
    """The backend entry points (hrt_update_glass with the materials) give the device solve's
    fluxes for a scene with covers."""
    a = _greenhouse(mode="device")
    b = _greenhouse(mode="backend")
    a.setSeed(3)
    b.setSeed(3)
    fa = a.runBand(["PAR", "NIR"])
    fb = b.runBand(["PAR", "NIR"])
    worst, _ = _flux_close(fb, fa, 1e-5)
    assert worst <= 1e-5, worst


def test_glass_errors(gpu):
    T, ty, ts = _mixed(seed=2, n_leaf=50, n_tri=50)
    gpu.update_geometry(T, ty, ts)
    gpu.build_accel()
    n = T.shape[0]
    ig = np.zeros((1, n, 2), np.int8)
    ig[0, :5] = 1
    bad_n = np.ones((1, n, 2), np.float32) * 0.5
    with pytest.raises(RuntimeError, match="refractive index"):
        gpu.update_glass(ig, bad_n, np.zeros((1, n, 2), np.float32))
    with pytest.raises(RuntimeError, match="geometry"):
        gpu.update_glass(ig[:, :-1], np.full((1, n - 1, 2), 1.5, np.float32), np.zeros((1, n - 1, 2), np.float32))
    gpu.update_glass(ig, np.full((1, n, 2), 1.5, np.float32), np.zeros((1, n, 2), np.float32))
    with pytest.raises(RuntimeError, match="sweep"):
        gpu.run_sweep(np.array([[0.0, 0.0, 1.0]]), np.ones((1, 2)), np.ones((1, 2)), np.full((n, 2), 0.1),
                      np.full((n, 2), 0.05), 4, 4, 1, 0)
    gpu.update_glass(None)


def test_device_matches_reference_estimator(oracle_mod):
    """Statistical parity of the device solve with the reference's Monte-Carlo estimator:
    K seeded device solves (Philox) against K seeded oracle solves that draw the reference's
    TEA-16 + LCG stream (OptiX8DeviceCode.cu:29-49): per primitive within 3 standard errors
    for >= 99 % of the primitives that carry flux, and in the canopy totals."""
    from test_oracle_reference_rng import K, canopy, check_statistical_parity

    rad, sc = canopy()
    scene = oracle_scene_for(rad, oracle_mod)

    def device(seed):
        rad.setSeed(seed)
        return rad.runBand("SW")

    seeds = range(300, 300 + K)
    dev = ensemble(device, seeds)
    with oracle_mod.reference_rng():
        ref = ensemble(lambda s: run_oracle(rad, ["SW"], oracle_mod, scene=scene, seed=s + 1000)[0], seeds)
    check_statistical_parity(dev, ref, sc.area)
