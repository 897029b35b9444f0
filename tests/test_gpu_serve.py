"""Served stream: continuous batching with device-resident scenes; every result equals the
same solve run alone, whether it ran alone, in a batch of its scene's requests, or in a
multi-scene group (small batches of different scenes traced by one persistent launch per pass)."""
import numpy as np
import pytest

from helios_gb300 import _hrt, scenes

pytestmark = pytest.mark.gpu


def _materials(sc):
    n = sc.n
    rho = np.tile(scenes.SERVED_RHO, (n, 1))
    tau = np.tile(scenes.SERVED_TAU, (n, 1))
    rho[sc.groups["ground"]] = 0.0
    tau[sc.groups["ground"]] = 0.0
    return rho, tau


def test_served_results_equal_alone(hrt_lib):
    sizes, lais, reqs = scenes.served_stream(n_requests=60, rate=200.0, n_scenes=5, n_min=2000, n_max=40000, seed=4)
    built = [scenes.mixed_canopy(int(sizes[k]), float(lais[k]), seed=k) for k in range(5)]
    srv = _hrt.Server(device=0, workers=4, hbm_budget=2 << 30)
    for k, sc in enumerate(built):
        rho, tau = _materials(sc)
        srv.add_scene(k, sc.T, sc.ptype, sc.twosided, rho, tau)
    for r in reqs:
        srv.submit(r["id"], r["scene"], r["arrival"], r["bands"], r["sun"], r["direct"], r["diffuse"], 64,
                   r["diffuse_rays"], 3, r["seed"], keep=True)
    srv.start()
    srv.wait()
    lat = []
    alone = _hrt.Context(0)
    cur = None
    for r in reqs[:20]:
        sc = built[r["scene"]]
        bl = int(r["bands"].sum())
        res = srv.result(r["id"], sc.n * bl)
        assert res["done"] >= res["admit"] >= res["arrival"] - 1e-3
        lat.append(res["done"] - res["arrival"])
        if cur != r["scene"]:
            alone.update_geometry(sc.T, sc.ptype, sc.twosided)
            alone.build_accel()
            cur = r["scene"]
        rho, tau = _materials(sc)
        desc = {"band_launch": r["bands"], "sources": [{"type": 0, "position": tuple(r["sun"])}],
                "source_flux": r["direct"], "rho": rho, "tau": tau, "diffuse_flux": r["diffuse"],
                "direct_rays": np.full(bl, 64), "diffuse_rays": np.full(bl, r["diffuse_rays"]),
                "depth": np.full(bl, 3), "emission": np.zeros(bl, np.uint8), "seed": r["seed"]}
        ref = alone.run_band(desc).reshape(-1)
        got = res["flux"]
        floor = 1e-3 * max(float(np.abs(ref).mean()), 1e-30)
        err = np.abs(got.astype(np.float64) - ref) / np.maximum(np.abs(ref), floor)
        assert err.max() <= 1e-5, (r["id"], err.max())
    st = srv.stats()
    assert st["builds"] >= 5
    # requests of a scene that were queued together ran as one batch
    assert st["batched_requests"] == len(reqs) and st["batches"] < len(reqs)
    srv.close()


def test_small_requests_of_different_scenes_share_one_sweep(hrt_lib):
    """Four small scenes, one request each, all arrived when the server starts: the first
    dispatch scan admits all four, and they run as one multi-scene sweep (each pass of all four
    scenes in one persistent launch); every result equals its solve alone."""
    built = [scenes.mixed_canopy(n, lai, seed=20 + k) for k, (n, lai) in
             enumerate(((2500, 1.5), (4000, 3.0), (6000, 0.8), (3000, 4.5)))]
    srv = _hrt.Server(device=0, workers=2, hbm_budget=2 << 30)
    for k, sc in enumerate(built):
        rho, tau = _materials(sc)
        srv.add_scene(k, sc.T, sc.ptype, sc.twosided, rho, tau)
    rng = np.random.default_rng(9)
    reqs = []
    for k in range(4):
        bands = np.array([1, k % 2, 1, 0], np.uint8)
        bl = int(bands.sum())
        r = {"id": k, "scene": k, "bands": bands, "sun": scenes.sun_direction(20 + 10 * k, 40 * k),
             "direct": rng.uniform(200, 900, bl), "diffuse": rng.uniform(20, 120, bl), "rays": 49 + 15 * k,
             "seed": 100 + k}
        srv.submit(r["id"], k, 0.0, bands, r["sun"], r["direct"], r["diffuse"], 36, r["rays"], 2, r["seed"], keep=True)
        reqs.append(r)
    srv.start()
    srv.wait()
    st = srv.stats()
    assert st["groups"] == 1 and st["grouped_batches"] == 4, st
    alone = _hrt.Context(0)
    for r in reqs:
        sc = built[r["scene"]]
        bl = int(r["bands"].sum())
        res = srv.result(r["id"], sc.n * bl)
        alone.update_geometry(sc.T, sc.ptype, sc.twosided)
        alone.build_accel()
        rho, tau = _materials(sc)
        desc = {"band_launch": r["bands"], "sources": [{"type": 0, "position": tuple(r["sun"])}],
                "source_flux": r["direct"], "rho": rho, "tau": tau, "diffuse_flux": r["diffuse"],
                "direct_rays": np.full(bl, 36), "diffuse_rays": np.full(bl, r["rays"]),
                "depth": np.full(bl, 2), "emission": np.zeros(bl, np.uint8), "seed": r["seed"]}
        ref = alone.run_band(desc).reshape(-1)
        floor = 1e-3 * max(float(np.abs(ref).mean()), 1e-30)
        err = np.abs(res["flux"].astype(np.float64) - ref) / np.maximum(np.abs(ref), floor)
        assert err.max() <= 1e-5, (r["id"], err.max())
    srv.close()


def test_oversize_request_rejected(hrt_lib):
    sc = scenes.mixed_canopy(4000, 2.0, seed=1)
    srv = _hrt.Server(device=0, workers=1, hbm_budget=1 << 20)  # 1 MB: no scene fits
    rho, tau = _materials(sc)
    srv.add_scene(0, sc.T, sc.ptype, sc.twosided, rho, tau)
    with pytest.raises(_hrt.HrtError):
        srv.submit(0, 0, 0.0, np.array([1, 0, 0, 0]), (0, 0, 1), [100.0], [10.0], 16, 16, 1, 1)
    srv.close()
