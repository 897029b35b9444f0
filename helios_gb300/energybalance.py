"""Energy balance: the step after the radiation solve, on the GPU.

Mirrors the user API of the reference's EnergyBalanceModel
(plugins/energybalance/include/EnergyBalanceModel.h; inputs and defaults of
plugins/energybalance/src/EnergyBalanceModel.cu:151-440 and EnergyBalanceModel.cpp:35-51)
over hrt_energy_balance, and couples it with RadiationModel on the device
(run_coupled: radiation -> surface temperature -> emission -> radiation, with the
temperatures resident in HBM between the solves).
"""
from __future__ import annotations

import math

import numpy as np

from . import _hrt
from .radiation import Context, HeliosRuntimeError, RadiationModel


def esat_Pa(T_K):
    """Saturated vapour pressure (Pa) at T (K) by the Clausius-Clapeyron fit the reference uses
    (EnergyBalanceModel.h:32-36), in FP32."""
    Tc = np.float32(T_K) - np.float32(273.15)
    return np.float32(611.0) * np.exp(np.float32(17.502) * Tc / (Tc + np.float32(240.97)), dtype=np.float32)


class EnergyBalanceModel:
    """Surface temperatures from the absorbed radiation of the bands added with
    addRadiationBand, air conditions and conductances read from primitive data."""

    OPTIONAL = ("boundarylayer_conductance_out", "vapor_pressure_deficit", "net_radiation_flux", "storage_flux")

    def __init__(self, context: Context, device: int = 0):
        self.context = context
        self.device = device
        self._ctx = None
        self.radiation_bands: list[str] = []
        self.output_prim_data: list[str] = []
        self.message_flag = True
        self.temperature_default = 300.0
        self.wind_speed_default = 1.0
        self.air_temperature_default = 300.0
        self.air_humidity_default = 0.5
        self.pressure_default = 101000.0
        self.gS_default = 0.0
        self.Qother_default = 0.0
        self.heatcapacity_default = 0.0
        self.surface_humidity_default = 1.0
        self.last_unconverged = 0

    @property
    def ctx(self) -> "_hrt.Context":
        if self._ctx is None:
            self._ctx = _hrt.Context(self.device)
        return self._ctx

    def disableMessages(self):
        self.message_flag = False

    def enableMessages(self):
        self.message_flag = True

    def addRadiationBand(self, band):
        for b in ([band] if isinstance(band, str) else list(band)):
            if b not in self.radiation_bands:
                self.radiation_bands.append(b)

    def optionalOutputPrimitiveData(self, label):
        if label not in self.OPTIONAL:
            raise HeliosRuntimeError(f"ERROR (EnergyBalanceModel::optionalOutputPrimitiveData): unknown output "
                                     f"primitive data {label}.")
        if label not in self.output_prim_data:
            self.output_prim_data.append(label)

    # ------------------------------------------------------------ inputs
    def _emissivity_bands(self):
        """Bands whose emissivity sets the emitted term: the emission-enabled ones when the
        radiation model recorded them (global data emission_enabled_<band>), else all."""
        g = self.context.global_data
        info = [b for b in self.radiation_bands if f"emission_enabled_{b}" in g]
        if info:
            return [b for b in self.radiation_bands if int(g.get(f"emission_enabled_{b}", 0)) == 1]
        return list(self.radiation_bands)

    def surface_arrays(self, uuids=None):
        """The per-primitive inputs of one solve (hrt_surface fields, FP32) with the reference's
        defaults and range checks, the absorbed radiation R and the initial temperature."""
        ctx = self.context
        n = ctx.getPrimitiveCount()
        uu = np.arange(n) if uuids is None else np.asarray(uuids, np.int64)
        if not self.radiation_bands:
            raise HeliosRuntimeError("ERROR (EnergyBalanceModel::run): No radiation bands were found.")
        R = np.zeros(uu.size, np.float32)
        for b in self.radiation_bands:
            a = ctx.primitive_array(f"radiation_flux_{b}", np.nan)[uu]
            if np.isnan(a).any():
                raise HeliosRuntimeError(f"ERROR (EnergyBalanceModel::run): No radiation was found in the context for "
                                         f"band {b}. Did you run the radiation model for this band?")
            R += a.astype(np.float32)

        def arr(label, default):
            return ctx.primitive_array(label, default)[uu]

        To = arr("temperature", self.temperature_default)
        To = np.where(To == 0, 300.0, To)
        Ta = arr("air_temperature", self.air_temperature_default)
        Ta = np.where(Ta < 250.0, self.air_temperature_default, Ta)
        hr = arr("air_humidity", self.air_humidity_default)
        hr = np.where((hr > 1.0) | (hr < 0.0), self.air_humidity_default, hr)
        Ta32 = Ta.astype(np.float32)
        ea = (hr.astype(np.float32) * esat_Pa(Ta32)).astype(np.float32)
        P = arr("air_pressure", self.pressure_default)
        P = np.where(P < 10000.0, self.pressure_default, P)
        ts = arr("twosided_flag", 1)
        nsides = np.where(ts == 0, 1, 2).astype(np.uint8)
        sided = arr("stomatal_sidedness", 0.0)
        ev = arr("evaporating_faces", np.nan)
        sided = np.where(np.isnan(ctx.primitive_array("stomatal_sidedness", np.nan)[uu]) & (ev == 2), 0.5, sided)
        sided = np.where(nsides == 2, sided, 0.0)
        gH_given = arr("boundarylayer_conductance", np.nan)
        U = arr("wind_speed", self.wind_speed_default)
        _, _, area = ctx.arrays()
        L = arr("object_length", 0.0)
        L = np.where(L == 0, np.sqrt(area[uu]), L)
        gH_calc = (np.float32(0.135) * np.sqrt((U / L).astype(np.float32)) * nsides.astype(np.float32)).astype(np.float32)
        self._calculated_gH = bool(np.isnan(gH_given).any())
        gH = np.where(np.isnan(gH_given), gH_calc, gH_given)
        gS = arr("moisture_conductance", self.gS_default)
        Qo = arr("other_surface_flux", self.Qother_default)
        cap = arr("heat_capacity", self.heatcapacity_default)
        hs = arr("surface_humidity", self.surface_humidity_default)
        eps = np.ones(uu.size)
        found = np.zeros(uu.size, bool)
        for b in self._emissivity_bands():
            e = arr(f"emissivity_{b}", np.nan)
            take = ~found & ~np.isnan(e)
            eps = np.where(take, e, eps)
            found |= ~np.isnan(e)
        f = lambda x: np.ascontiguousarray(x, np.float32)
        surf = {"air_temperature": f(Ta), "air_vapor_pressure": f(ea), "air_pressure": f(P), "bl_conductance": f(gH),
                "moisture_conductance": f(gS), "emissivity": f(eps), "other_flux": f(Qo), "heat_capacity": f(cap),
                "surface_humidity": f(hs), "stomatal_sidedness": f(sided), "nsides": nsides,
                "temperature_default": self.temperature_default}
        return surf, R, f(To), uu

    # ------------------------------------------------------------ solve
    def run(self, dt: float = 0.0, UUIDs=None):
        """EnergyBalanceModel::run: solve the surface temperatures and write temperature,
        sensible_flux, latent_flux (and the optional outputs) as primitive data."""
        surf, R, To, uu = self.surface_arrays(UUIDs)
        surf["dt"] = float(dt)
        T, out = self.ctx.energy_balance(surf, net_radiation=R, temperature=To, outputs=True)
        self.last_unconverged = self.ctx.last_stats()["eb_unconverged"]
        self.write_outputs(uu, T, out, surf)
        return T

    def write_outputs(self, uu, T, out, surf):
        ctx = self.context
        ctx.setPrimitiveData(uu, "temperature", T.astype(np.float64))
        if out is not None:
            ctx.setPrimitiveData(uu, "sensible_flux", out[:, 0].astype(np.float64))
            ctx.setPrimitiveData(uu, "latent_flux", out[:, 1].astype(np.float64))
        labels = list(self.output_prim_data)
        if getattr(self, "_calculated_gH", False) and "boundarylayer_conductance_out" not in labels:
            labels.append("boundarylayer_conductance_out")
        for lab in labels:
            if lab == "boundarylayer_conductance_out":
                ctx.setPrimitiveData(uu, lab, surf["bl_conductance"].astype(np.float64))
            elif out is not None and lab == "vapor_pressure_deficit":
                ctx.setPrimitiveData(uu, lab, out[:, 4].astype(np.float64))
            elif out is not None and lab == "net_radiation_flux":
                ctx.setPrimitiveData(uu, lab, out[:, 3].astype(np.float64))
            elif out is not None and lab == "storage_flux":
                ctx.setPrimitiveData(uu, lab, out[:, 2].astype(np.float64))


def run_coupled(radiation: RadiationModel, energy: EnergyBalanceModel, band_labels, max_iterations: int = 20,
                tolerance: float = 1e-3):
    """Radiation and energy balance coupled on the device (hrt_run_coupled): runBand over
    band_labels with the current temperatures, the energy balance on its fluxes, the new
    temperatures emitted by the next runBand, until no temperature moves by more than
    tolerance (K).  The energy balance's bands must be the launched bands.  Writes
    radiation_flux_<band> of the last solve and temperature; returns the iterations run."""
    labels = [band_labels] if isinstance(band_labels, str) else list(band_labels)
    if sorted(energy.radiation_bands) != sorted(labels):
        raise HeliosRuntimeError("ERROR (run_coupled): the energy balance bands must be the launched bands.")
    ctx = radiation.context
    n = ctx.getPrimitiveCount()
    if radiation._geom_n != n:
        radiation.updateGeometry()
    for b in labels:  # the surface inputs need radiation_flux_<band>; the coupled solve recomputes them
        if np.isnan(ctx.primitive_array(f"radiation_flux_{b}", np.nan)).any():
            ctx.setPrimitiveData(np.arange(n), f"radiation_flux_{b}", np.zeros(n))
    for b in radiation.bands:
        ctx.setGlobalData("emission_enabled_" + b, 1 if radiation.bands[b].emissionFlag else 0)
    surf, _, To, uu = energy.surface_arrays()
    desc = radiation.solve_description(labels)
    desc["temperature"] = To
    flux, T, it = radiation.ctx.run_coupled(desc, surf, max_iterations, tolerance)
    for i, b in enumerate(desc["band_labels"]):
        ctx.setPrimitiveData(uu, "radiation_flux_" + b, flux[:, i].astype(np.float64))
    energy.write_outputs(uu, T, None, surf)
    energy.last_unconverged = radiation.ctx.last_stats()["eb_unconverged"]
    if radiation.auto_seed:
        radiation.seed = (radiation.seed + 0x9E3779B9) & 0xFFFFFFFF
    return it
