"""Energy balance on the GPU: the reference's energy balance tests, the device solve against
the FP32 oracle, and the coupled radiation / energy balance loop against the same loop run
step by step on the oracle."""
import math

import numpy as np
import pytest

from helios_gb300 import scenes
from helios_gb300.energybalance import EnergyBalanceModel, run_coupled
from helios_gb300.radiation import Context, RadiationModel

import scenarios
from helpers import oracle_scene_for, oracle_solve

pytestmark = pytest.mark.gpu

T_ATOL = 1e-3  # K: device vs oracle surface temperature


@pytest.mark.parametrize("name", scenarios.ENERGY)
def test_energy_balance_known_answers_on_gpu(name):
    def run_eb(model, dt):
        model.run(dt)
    res = getattr(scenarios, name)(run_eb)
    absn = [r[0] for r in res if r[2] == 0.0]
    assert not scenarios.check(res, abs_tol_names=absn), scenarios.check(res, abs_tol_names=absn)


def _random_surface(n, seed):
    rng = np.random.default_rng(seed)
    Ta = rng.uniform(270.0, 315.0, n).astype(np.float32)
    surf = {"air_temperature": Ta,
            "air_vapor_pressure": (rng.uniform(0.1, 0.9, n) * 611.0 * np.exp(17.502 * (Ta - 273.15) / (Ta - 273.15 + 240.97))).astype(np.float32),
            "air_pressure": rng.uniform(9.0e4, 1.02e5, n).astype(np.float32),
            "bl_conductance": rng.uniform(0.0, 2.0, n).astype(np.float32),
            "moisture_conductance": np.where(rng.random(n) < 0.3, 0.0, rng.uniform(0.0, 0.5, n)).astype(np.float32),
            "emissivity": rng.uniform(0.8, 1.0, n).astype(np.float32),
            "other_flux": rng.uniform(-50.0, 150.0, n).astype(np.float32),
            "heat_capacity": rng.uniform(0.0, 5000.0, n).astype(np.float32),
            "surface_humidity": rng.uniform(0.5, 1.0, n).astype(np.float32),
            "stomatal_sidedness": rng.uniform(0.0, 0.5, n).astype(np.float32),
            "nsides": rng.integers(1, 3, n).astype(np.uint8), "dt": 60.0, "temperature_default": 300.0}
    R = rng.uniform(100.0, 1500.0, n).astype(np.float32)
    To = (Ta + rng.uniform(-5.0, 15.0, n)).astype(np.float32)
    return surf, R, To


def test_energy_balance_vs_oracle(oracle_mod):
    """Temperatures within 1e-3 K of the FP32 oracle (the same secant steps; only expf may
    round differently), fluxes within 1e-3 relative."""
    from helios_gb300 import _hrt
    ctx = _hrt.Context(0)
    for seed in (1, 2):
        surf, R, To = _random_surface(20000, seed)
        T1, o1 = ctx.energy_balance(surf, net_radiation=R, temperature=To, outputs=True)
        T2, o2, bad = oracle_mod.energy_balance(surf, R, To)
        assert np.abs(T1 - T2).max() <= T_ATOL
        assert ctx.last_stats()["eb_unconverged"] == bad
        # fluxes follow T: within 1e-3 relative or 0.05 W/m^2 (storage amplifies T by C / dt)
        assert np.allclose(o1[:, :4], o2[:, :4], rtol=1e-3, atol=5e-2)
        assert np.allclose(o1[:, 4], o2[:, 4], rtol=1e-3, atol=1e-6)


def _coupled_scene(seed=0, n_leaves=1500):
    sc = scenes.homogeneous_canopy(n_leaves=n_leaves, leaf=0.1, domain=3.0, zlo=0.5, zhi=2.0, seed=seed)
    ctx = Context()
    ctx.addScene(sc)
    lv = sc.groups["leaves"]
    n = sc.n
    ctx.setPrimitiveData(lv, "reflectivity_SW", np.full(lv.size, 0.15))
    ctx.setPrimitiveData(lv, "transmissivity_SW", np.full(lv.size, 0.10))
    ctx.setPrimitiveData(np.arange(n), "emissivity_LW", np.full(n, 0.96))
    ctx.setPrimitiveData(np.arange(n), "temperature", np.full(n, 295.0))
    ctx.setPrimitiveData(np.arange(n), "air_temperature", np.full(n, 298.0))
    ctx.setPrimitiveData(np.arange(n), "moisture_conductance", np.full(n, 0.2))
    ctx.setPrimitiveData(np.arange(n), "object_length", np.full(n, 0.1))
    rad = RadiationModel(ctx)
    rad.enforcePeriodicBoundary("xy")
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(30, 0))
    rad.addRadiationBand("SW")
    rad.disableEmission("SW")
    rad.setSourceFlux(sun, "SW", 800.0)
    rad.setDiffuseRadiationFlux("SW", 100.0)
    rad.addRadiationBand("LW")
    rad.setDiffuseRadiationFlux("LW", 350.0)
    for b in ("SW", "LW"):
        rad.setDirectRayCount(b, 25)
        rad.setDiffuseRayCount(b, 64)
        rad.setScatteringDepth(b, 2)
    eb = EnergyBalanceModel(ctx)
    eb.disableMessages()
    eb.addRadiationBand(["SW", "LW"])
    return rad, eb, ctx


def test_coupled_loop_vs_oracle_loop(oracle_mod):
    """hrt_run_coupled (temperatures resident on the device between solves) against the same
    fixed-point loop on the oracle: runBand with the current temperatures, the energy balance
    on the sum of its band fluxes, repeated the same number of times."""
    rad, eb, ctx = _coupled_scene()
    rad.setSeed(7)
    it = run_coupled(rad, eb, ["SW", "LW"], max_iterations=30, tolerance=1e-3)
    assert 2 <= it < 30
    T_gpu = ctx.primitive_array("temperature", np.nan).astype(np.float32)
    rad2, eb2, ctx2 = _coupled_scene()
    n = ctx2.getPrimitiveCount()
    for b in ("SW", "LW"):  # surface inputs only; the loop below computes the fluxes
        ctx2.setPrimitiveData(np.arange(n), "radiation_flux_" + b, np.zeros(n))
    surf, _, To, _ = eb2.surface_arrays()
    sc = oracle_scene_for(rad2, oracle_mod)
    T = To.copy()
    for _ in range(it):
        desc = rad2.solve_description(["SW", "LW"], seed=7)
        desc["temperature"] = T
        flux, _ = sc.run_band(oracle_solve(desc))
        f32 = flux.astype(np.float32)
        R = np.zeros(f32.shape[0], np.float32)
        for b in range(f32.shape[1]):
            R += f32[:, b]
        T, _, _ = oracle_mod.energy_balance(surf, R, T)
    assert np.abs(T_gpu - T).max() <= 5e-3
    assert np.abs(T_gpu - 298.0).max() < 40.0


def test_coupled_matches_host_loop():
    """The coupled solve equals runBand + EnergyBalanceModel.run repeated from the host."""
    rad, eb, ctx = _coupled_scene(seed=1, n_leaves=800)
    rad.setSeed(3)
    it = run_coupled(rad, eb, ["SW", "LW"], max_iterations=6, tolerance=0.0)
    assert it == 6
    T_dev = ctx.primitive_array("temperature", np.nan)
    rad2, eb2, ctx2 = _coupled_scene(seed=1, n_leaves=800)
    n = ctx2.getPrimitiveCount()
    for _ in range(6):
        rad2.setSeed(3)
        rad2.runBand(["SW", "LW"])
        eb2.run()
    T_host = ctx2.primitive_array("temperature", np.nan)
    assert np.abs(T_dev - T_host).max() <= 1e-3
    assert n == T_dev.size
