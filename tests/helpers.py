"""Shared helpers: run one runBand through the oracle or the GPU engine."""
from __future__ import annotations

import math

import numpy as np


def rotation_np(r):
    """Row-major 3x3 rotation of rect/disk sources (same formula as hrt_source_rotation)."""
    sx, cx = math.sin(r[0]), math.cos(r[0])
    sy, cy = math.sin(r[1]), math.cos(r[1])
    sz, cz = math.sin(r[2]), math.cos(r[2])
    return np.array([cz * cy, cz * sy * sx - sz * cx, cz * sy * cx + sz * sx,
                     sz * cy, sz * sy * sx + cz * cx, sz * sy * cx - cz * sx,
                     -sy, cy * sx, cy * cx], np.float32)


def oracle_solve(desc: dict, rotation=rotation_np) -> dict:
    """Convert a RadiationModel.solve_description() dict to the oracle's solve dict."""
    srcs = desc["sources"]
    d = {k: desc[k] for k in ("band_launch", "source_flux", "rho", "tau", "diffuse_flux", "diffuse_ext",
                              "diffuse_norm", "diffuse_peak", "prague", "direct_rays", "diffuse_rays", "depth",
                              "emission", "eps", "temperature", "seed")}
    d["scatter_tolerance"] = desc.get("scatter_tolerance", 0.0)
    for k in ("is_glass", "glass_n", "glass_kl", "cameras", "camera_sky"):
        d[k] = desc.get(k)
    d["source_type"] = np.array([s["type"] for s in srcs], np.int32)
    d["source_pos"] = np.array([s["position"] for s in srcs], np.float32)
    d["source_width"] = np.array([s["width"] for s in srcs], np.float32)
    d["source_rot"] = np.stack([rotation(s.get("rotation", (0, 0, 0))) for s in srcs]).astype(np.float32)
    return d


def oracle_scene_for(rad, oracle_mod):
    T, ty, ts = rad.geometry_arrays()
    bb = rad._bbox_faces()
    return oracle_mod.OracleScene(T, ty, ts, bb, rad.periodic, rad.voxel_lad(), rad.context.mask_arrays())


def run_oracle(rad, labels, oracle_mod, scene=None, seed=None, threads=0):
    """Flux [n, Bl] (float64) of one runBand computed by the FP64 oracle."""
    desc = rad.solve_description(labels, seed=seed)
    sc = scene or oracle_scene_for(rad, oracle_mod)
    flux, stats = sc.run_band(oracle_solve(desc), threads=threads)
    return flux, stats


def beer_diffuse(lai, n=50):
    """Hemispherical integral of canopy interception under isotropic sky (selfTest.cpp:1453-1462)."""
    dth = 0.5 * math.pi / n
    acc = 0.0
    for i in range(n):
        th = (i + 0.5) * dth
        acc += 2.0 * (1.0 - math.exp(-0.5 * lai / math.cos(th))) * math.cos(th) * math.sin(th) * dth
    return acc


def view_factor_parallel(a, b, c):
    """F12 of two directly opposed a x b rectangles at distance c (selfTest.cpp:685-686)."""
    X, Y = a / c, b / c
    X2, Y2 = X * X, Y * Y
    return 2.0 / (math.pi * X * Y) * (math.log(math.sqrt((1 + X2) * (1 + Y2) / (1 + X2 + Y2)))
                                      + X * math.sqrt(1 + Y2) * math.atan(X / math.sqrt(1 + Y2))
                                      + Y * math.sqrt(1 + X2) * math.atan(Y / math.sqrt(1 + X2))
                                      - X * math.atan(X) - Y * math.atan(Y))


def glass_ref(cos_theta, n, KL):
    """Single-sheet (tau, rho, alpha) in the angle form the reference's glass tests use as
    their independent check (selfTest.cpp:9556-9591): Fresnel r_s = sin^2(t_r - t) /
    sin^2(t_r + t), r_p = tan^2(t_r - t) / tan^2(t_r + t), Bouguer exp(-KL / cos t_r) and
    incoherent multiple reflections; float64 here."""
    c = min(1.0, max(1e-4, cos_theta))
    th = math.acos(c)
    st = math.sin(th) / n
    ctr = math.sqrt(max(0.0, 1.0 - st * st))
    tr = math.asin(min(1.0, st))
    if th < 1e-3:
        r_s = r_p = ((n - 1.0) / (n + 1.0)) ** 2
    else:
        r_s = math.sin(tr - th) ** 2 / max(1e-12, math.sin(tr + th) ** 2)
        r_p = math.tan(tr - th) ** 2 / max(1e-12, math.tan(tr + th) ** 2)
    ta = math.exp(-KL / max(1e-4, ctr)) if KL > 0 else 1.0
    tau = rho = 0.0
    for r in (r_s, r_p):
        den = max(1e-6, 1.0 - (r * ta) ** 2)
        ti = ta * (1.0 - r) ** 2 / den
        tau += 0.5 * ti
        rho += 0.5 * r * (1.0 + ta * ti)
    tau, rho = min(1.0, max(0.0, tau)), min(1.0, max(0.0, rho))
    return tau, rho, max(0.0, 1.0 - tau - rho)


def run_oracle_cameras(rad, labels, oracle_mod, seed=None):
    """(flux, {camera label: dict(pixels, labels, depths)}) of one runBand by the oracle."""
    desc = rad.solve_description(labels, seed=seed)
    sc = oracle_scene_for(rad, oracle_mod)
    flux, stats = sc.run_band(oracle_solve(desc))
    cams = dict(zip(desc.get("camera_labels", []), stats.get("cameras", [])))
    return flux, cams


def run_device_cameras(rad, labels, seed):
    """(flux, {camera label: dict(pixels, labels, depths)}) of one runBand on the device."""
    rad.setSeed(seed)
    flux = rad.runBand(labels)
    cams = {}
    for label, cam in rad.cameras.items():
        if cam["labels"] is None:
            continue
        W, H = cam["props"]["camera_resolution"]
        bands = [b for b in sorted(rad.bands) if b in labels]
        pix = np.stack([cam["pixels"][b].reshape(H, W) for b in bands], axis=-1)
        cams[label] = {"pixels": pix, "labels": cam["labels"].reshape(H, W), "depths": cam["depths"].reshape(H, W)}
    return flux, cams


def ensemble(solve, seeds):
    """[K, n] fluxes of solve(seed) over the seeds (first band)."""
    return np.stack([np.asarray(solve(s), np.float64)[:, 0] for s in seeds])


def z_scores(a, b, floor_frac=1e-3):
    """Per-primitive difference of the ensemble means of a and b [K, n] in units of its
    standard error; primitives whose mean flux is below floor_frac of the average, or whose
    samples do not vary, are left out."""
    ka, kb = a.shape[0], b.shape[0]
    ma, mb = a.mean(0), b.mean(0)
    se = np.sqrt(a.var(0, ddof=1) / ka + b.var(0, ddof=1) / kb)
    keep = (np.abs(0.5 * (ma + mb)) > floor_frac * np.abs(0.5 * (ma + mb)).mean()) & (se > 0)
    return (ma - mb)[keep] / se[keep]
