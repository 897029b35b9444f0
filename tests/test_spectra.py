"""Spectral radiative properties in the mirror (RadiationModel::updateRadiativeProperties,
RadiationModel.cpp:1998-2700): a primitive's `reflectivity_spectrum` / `transmissivity_spectrum`
name global (wavelength, value) data, averaged over each band's waveband -- weighted by the
source's spectrum when it has one (integrateSpectrum, :1463-1505), flat otherwise (:1507-1538,
divided by the band width at :2450) -- unless a band constant other than the default is set.
CPU only: the rule itself, and an absorbed-flux known answer on the oracle."""
import numpy as np
import pytest

from helios_gb300.radiation import Context, RadiationModel, _spectrum_over_band

from helpers import run_oracle

# the reference test's leaf and solar spectra (selfTest.cpp:2355-2410)
RHO = [(400, 0.05), (500, 0.10), (600, 0.08), (700, 0.45), (800, 0.50)]
TAU = [(400, 0.02), (500, 0.05), (600, 0.04), (700, 0.40), (800, 0.45)]
SUN = [(400, 1.5), (500, 2.0), (600, 1.8), (700, 1.2), (800, 1.0), (900, 0.8)]


def _segments(spec, w1, w2, with_source):
    """The object-spectrum segments integrateSpectrum sums for [w1, w2]."""
    xs = [x for x, _ in spec]
    istart, iend = (0 if with_source else 1), len(xs) - 1
    for i in range(len(xs) - 1):
        if xs[i] <= w1 < xs[i + 1]:
            istart = i
        if xs[i] <= w2 < xs[i + 1]:
            iend = i + 1
            break
    return range(istart, iend)


def _expected(spec, w1, w2, source=None):
    """FP64 value of the same rule, written out independently."""
    xs, ys = np.array([x for x, _ in spec], float), np.array([y for _, y in spec], float)
    segs = list(_segments(spec, w1, w2, source is not None))
    if source is None:
        return sum(0.5 * (ys[i] + ys[i + 1]) * (xs[i + 1] - xs[i]) for i in segs) / (w2 - w1)
    sx, sy = np.array([x for x, _ in source], float), np.array([y for _, y in source], float)
    S = np.interp(xs, sx, sy)  # linear, clamped at the ends (helios::interp1)
    num = sum(0.5 * (ys[i] * S[i] + ys[i + 1] * S[i + 1]) * (xs[i + 1] - xs[i]) for i in segs)
    den = sum(0.5 * (S[i] + S[i + 1]) * (xs[i + 1] - xs[i]) for i in segs)
    return num / den


@pytest.mark.parametrize("w1,w2", [(400, 700), (700, 900), (450, 650), (400, 800)])
@pytest.mark.parametrize("weighted", [False, True])
def test_band_average_rule(w1, w2, weighted):
    src = SUN if weighted else None
    got = _spectrum_over_band(RHO, w1, w2, src)
    if not weighted:
        got /= (w2 - w1)
    assert got == pytest.approx(_expected(RHO, w1, w2, src), rel=2e-6)


def test_flat_spectrum_equals_constant_with_a_source_spectrum():
    flat = [(w, 0.3) for w in range(380, 905, 5)]
    assert _spectrum_over_band(flat, 400, 700, SUN) == pytest.approx(0.3, rel=1e-6)


def _patch_model(spectral=True, constant=None, bounds=(400, 700), sun_spectrum=True):
    ctx = Context()
    p = ctx.addPatch((0, 0, 0), (1, 1))
    ctx.setPrimitiveData(p, "twosided_flag", 0)
    ctx.setGlobalData("leaf_rho", RHO)
    ctx.setGlobalData("leaf_tau", TAU)
    ctx.setGlobalData("solar", SUN)
    if spectral:
        ctx.setPrimitiveData(p, "reflectivity_spectrum", "leaf_rho")
        ctx.setPrimitiveData(p, "transmissivity_spectrum", "leaf_tau")
    if constant is not None:
        ctx.setPrimitiveData(p, "reflectivity_VIS", constant)
    rad = RadiationModel(ctx)
    rad.addRadiationBand("VIS", *bounds) if bounds else rad.addRadiationBand("VIS")
    rad.disableEmission("VIS")
    sun = rad.addCollimatedRadiationSource((0, 0, 1))
    if sun_spectrum:
        rad.setSourceSpectrum(sun, "solar")
    rad.setSourceFlux(sun, "VIS", 1000.0)
    rad.setDirectRayCount("VIS", 100)
    rad.setScatteringDepth("VIS", 0)
    return rad


def test_materials_follow_the_reference_precedence():
    rho, tau, _ = _patch_model()._materials(["VIS"], 1)
    assert rho[0, 0, 0] == pytest.approx(_expected(RHO, 400, 700, SUN), rel=2e-6)
    assert tau[0, 0, 0] == pytest.approx(_expected(TAU, 400, 700, SUN), rel=2e-6)
    rho, _, _ = _patch_model(sun_spectrum=False)._materials(["VIS"], 1)
    assert rho[0, 0, 0] == pytest.approx(_expected(RHO, 400, 700), rel=2e-6)
    rho, _, _ = _patch_model(constant=0.2)._materials(["VIS"], 1)  # a band constant wins
    assert rho[0, 0, 0] == pytest.approx(0.2)
    rho, tau, _ = _patch_model(bounds=None)._materials(["VIS"], 1)  # no waveband: defaults
    assert rho[0, 0, 0] == 0.0 and tau[0, 0, 0] == 0.0


def test_spectral_patch_absorbs_its_band_share(oracle_mod):
    """A one-sided horizontal patch alone under a zenith sun of 1000 W/m^2, one scattering
    iteration (its reflected and transmitted shares leave the scene; with depth 0 runBand would
    add them back, RadiationModel.cpp:4652): the flux is 1000 (1 - rho_band - tau_band) with the
    band values of the rule."""
    rad = _patch_model()
    rad.setScatteringDepth("VIS", 1)
    f, _ = run_oracle(rad, ["VIS"], oracle_mod, seed=3)
    exp = 1000.0 * (1.0 - _expected(RHO, 400, 700, SUN) - _expected(TAU, 400, 700, SUN))
    assert f[0, 0] == pytest.approx(exp, rel=1e-5)
