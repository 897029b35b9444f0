"""GPU parity for native disks, turbid-medium voxels and the FP64 scattering residual
(the deep-scattering stress workload, scaled down so the oracle finishes in seconds).

Bit-exact: device records/BVH, generated ray sets (disk concentric map, voxel
interior points and isotropic pairs) and hit IDs through voxels (free-path draws
keyed by ray and voxel).  Flux: per-primitive relative error <= 1e-4 against the
FP64 oracle, and the same number of scattering iterations under the residual stop.
"""
import numpy as np
import pytest

from helios_gb300 import _hrt, scenes
from helios_gb300.radiation import Context, HeliosRuntimeError, RadiationModel

import scenarios
from helpers import oracle_solve, oracle_scene_for, run_oracle

pytestmark = pytest.mark.gpu

FLUX_RTOL = 1e-4  # per-primitive relative flux error vs the FP64 oracle


def _flux_close(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    floor = 1e-3 * max(float(np.abs(ref).mean()), 1e-30)
    return float((np.abs(got - ref) / np.maximum(np.abs(ref), floor)).max())


def _stress(n_tri=4000, n_patch=700, n_disk=700, vox_div=6, seed=2):
    return scenes.deep_scatter(n_tri=n_tri, n_patch=n_patch, n_disk=n_disk, vox_div=vox_div, domain=3.0, height=1.5,
                               seed=seed)


def _stress_model(sc, depth=20, tol=0.0, mode="device", rays=(16, 36)):
    ctx = Context()
    ctx.addScene(sc)
    n = ctx.getPrimitiveCount()
    leaves = np.arange(1, n)
    ctx.setPrimitiveData(leaves, "reflectivity_NIR", np.full(n - 1, 0.45))
    ctx.setPrimitiveData(leaves, "transmissivity_NIR", np.full(n - 1, 0.40))
    rad = RadiationModel(ctx, mode=mode)
    rad.enforcePeriodicBoundary("xy")
    rad.addRadiationBand("NIR")
    rad.disableEmission("NIR")
    rad.setDirectRayCount("NIR", rays[0])
    rad.setDiffuseRayCount("NIR", rays[1])
    rad.setDiffuseRadiationFlux("NIR", 100.0)
    rad.setScatteringDepth("NIR", depth)
    rad.setScatteringResidualTolerance(tol)
    src = rad.addCollimatedRadiationSource(scenes.sun_direction(35.0, 20.0))
    rad.setSourceFlux(src, "NIR", 400.0)
    return rad


@pytest.fixture(scope="module")
def gpu(hrt_lib):
    return _hrt.Context(0)


def test_bvh_bit_exact_with_disks_and_voxels(gpu, oracle_mod):
    sc = _stress()
    gpu.update_geometry(sc.T, sc.ptype, sc.twosided, voxel_lad=sc.lad)
    gpu.build_accel()
    c1, p1, n1 = gpu.bvh()
    c2, p2, n2 = oracle_mod.OracleScene(sc.T, sc.ptype, sc.twosided, voxel_lad=sc.lad).bvh()
    assert np.array_equal(c1, c2)
    assert np.array_equal(p1, p2)
    assert np.array_equal(n1[:, 12:14], n2[:, 12:14])
    assert np.array_equal(n1[:, :12].view(np.float32), n2[:, :12].view(np.float32))


@pytest.mark.parametrize("kind,face", [(0, 0), (1, 1), (1, 0)])
def test_ray_sets_bit_exact_disks_voxels(gpu, oracle_mod, kind, face):
    sc = _stress(n_tri=300, n_patch=300, n_disk=300, vox_div=4)
    gpu.update_geometry(sc.T, sc.ptype, sc.twosided, voxel_lad=sc.lad)
    gpu.build_accel()
    osc = oracle_mod.OracleScene(sc.T, sc.ptype, sc.twosided, voxel_lad=sc.lad)
    sun = scenes.sun_direction(30, 0)
    rpp = 100 if kind == 0 else 324
    o1, d1 = gpu.gen_rays(kind, 99, 3, rpp, face, sun)
    o2, d2 = osc.gen_rays(kind, 99, 3, rpp, face, sun)
    assert np.array_equal(o1, o2)
    assert np.array_equal(d1, d2)
    # voxel origins lie inside their box; disk origins inside their radius
    nr = o1.shape[0] // sc.n
    vox = sc.groups["voxels"]
    T = sc.T[vox].astype(np.float64)
    c = T[:, [3, 7, 11]]
    h = 0.5 * np.abs(T[:, [0, 5, 10]])
    ov = o1.reshape(sc.n, nr, 3)[vox]
    assert np.all(np.abs(ov - c[:, None, :]) <= h[:, None, :] * (1 + 1e-6))
    dk = sc.groups["disks"]
    od = o1.reshape(sc.n, nr, 3)[dk] - sc.T[dk][:, [3, 7, 11]][:, None, :]
    assert np.all(np.linalg.norm(od, axis=-1) <= 0.02 * (1 + 1e-5))


def test_hit_ids_exact_through_voxels(gpu, oracle_mod):
    sc = _stress(seed=5)
    gpu.update_geometry(sc.T, sc.ptype, sc.twosided, voxel_lad=sc.lad)
    gpu.build_accel()
    osc = oracle_mod.OracleScene(sc.T, sc.ptype, sc.twosided, voxel_lad=sc.lad)
    rng = np.random.default_rng(8)
    n = 150000
    o = np.stack([rng.uniform(-0.5, 3.5, n), rng.uniform(-0.5, 3.5, n), rng.uniform(-0.5, 2.0, n)], 1)
    d = scenes.uniform_sphere(rng, n)
    h1, t1, f1 = gpu.trace_rays(o.astype(np.float32), d.astype(np.float32))
    h2, t2, f2, _ = osc.trace(o, d)
    assert (np.isin(h1, sc.groups["voxels"])).mean() > 0.05
    assert np.array_equal(h1, h2)
    assert np.array_equal(t1[h1 >= 0], t2[h2 >= 0])
    assert np.array_equal(f1, f2)
    assert gpu.device_status() == 0


@pytest.mark.parametrize("tol", [0.0, 1e-3])
def test_stress_flux_vs_oracle(oracle_mod, tol):
    """Scaled-down deep-scatter stress: triangles, patches, disks and a voxel grid,
    periodic, NIR (rho 0.45, tau 0.40), depth 20 -- full depth, and the residual stop."""
    sc = _stress()
    rad = _stress_model(sc, depth=20, tol=tol)
    rad.setSeed(21)
    got = rad.runBand("NIR")
    ref, st = run_oracle(rad, ["NIR"], oracle_mod, seed=21)
    assert rad.last_stats["iterations"] == st["iterations"]
    assert (st["iterations"] == 20) == (tol == 0.0)
    assert rad.last_stats["rays"] == st["rays"]
    worst = _flux_close(got, ref)
    assert worst <= FLUX_RTOL, worst


def test_stress_variants_agree(oracle_mod):
    """On a scene with voxels every diffuse-kernel variant (persistent over binary nodes,
    one ray per thread, persistent over compressed 4-wide nodes) gives the oracle's fluxes
    and ray count, and the statistics launches count on the forced variant's tree (the
    binary and 4-wide node-visit counts differ)."""
    sc = _stress()
    visits = {}
    for variant in (1, 3, 4):
        rad = _stress_model(sc, depth=6)
        rad.ctx.set_tuning(16 + variant)
        rad.setSeed(23)
        got = rad.runBand("NIR")
        rays = rad.last_stats["rays"]
        rad.ctx.set_measure(1)
        rad.setSeed(23)
        rad.runBand("NIR")
        visits[variant] = rad.ctx.get_measure()["node_visits"]
        rad.ctx.set_measure(0)
        ref, st = run_oracle(rad, ["NIR"], oracle_mod, seed=23)
        assert rays == st["rays"]
        worst = _flux_close(got, ref)
        assert worst <= FLUX_RTOL, (variant, worst)
        assert rad.ctx.device_status() == 0
    assert visits[1] > 0 and visits[4] > 0 and visits[1] != visits[4]


def test_stress_backend_sequence_matches_device():
    """The RayTracingBackend-shaped call sequence gives the device solve's numbers on a
    scene with disks and voxels (fixed depth: that sequence has no residual stop)."""
    sc = _stress(n_tri=2000, n_patch=300, n_disk=300, vox_div=4)
    a = _stress_model(sc, depth=4, mode="device")
    b = _stress_model(sc, depth=4, mode="backend")
    a.setSeed(4)
    b.setSeed(4)
    fa = a.runBand("NIR")
    fb = b.runBand("NIR")
    assert _flux_close(fb, fa) <= 1e-5


@pytest.mark.parametrize("name", ["disk_view_factor", "voxel_beer", "voxel_isothermal"])
def test_known_answers_on_gpu(name):
    def run(rad, labels, seed):
        rad.setSeed(seed)
        return rad.runBand(labels)
    res = getattr(scenarios, name)(run)
    assert not scenarios.check(res), scenarios.check(res)


def test_gray_voxel_cavity_on_gpu():
    def run(rad, labels, seed):
        rad.setSeed(seed)
        return rad.runBand(labels)
    res = scenarios.voxel_isothermal(run, eps=0.6)
    assert not scenarios.check(res), scenarios.check(res)


def test_voxel_errors(hrt_lib):
    v = scenes.voxel_grid((0, 0, 0), (1, 1, 1), (2, 2, 2), 1.0)
    g = _hrt.Context(0)
    with pytest.raises(_hrt.HrtError):
        g.update_geometry(v.T, v.ptype, v.twosided)  # voxels without leaf area density
    with pytest.raises(_hrt.HrtError):
        g.update_geometry(v.T, v.ptype, v.twosided, voxel_lad=np.full(v.n, -1.0))
    g.update_geometry(v.T, v.ptype, v.twosided, voxel_lad=v.lad)
    g.build_accel()
    with pytest.raises(_hrt.HrtError):  # the batched sweep does not trace voxels
        g.run_sweep(np.array([[0.0, 0.0, 1.0]]), np.ones((1, 1)), np.zeros((1, 1)), np.zeros((v.n, 1)),
                    np.zeros((v.n, 1)), 16, 16, 1, 0)
    ctx = Context()
    ctx.addVoxel((0, 0, 0), (1, 1, 1))
    rad = RadiationModel(ctx)
    rad.addRadiationBand("SW")
    with pytest.raises(HeliosRuntimeError):
        rad.setScatteringResidualTolerance(-1.0)
