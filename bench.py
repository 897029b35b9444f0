"""Benchmark: rays/s and solves/s of the radiation solve on one GB300.

Workload (default): the orchard triangle mesh — 200 trees on a 20 x 10 grid at
5 m, 5,000 equilateral 3 cm triangular leaves per tree in ellipsoidal crowns
(1.0 M triangles), 3 bands (PAR rho .08 tau .05, NIR rho .45 tau .40, LW eps .96
with leaf T ~ N(25, 2^2) C), sun at zenith 30 deg, 100 direct and 200 diffuse
(15 x 15 = 225) rays per primitive, scattering depth 5.  Synthetic, seeded
(seed 0).  One step = one full runBand (direct + primary diffuse + 5 scattering
passes) over the resident scene.

Arms:
  (default)          libhrt on cuda:0; `value` = device-resident rays/s, `e2e` =
                     rays/s through the C ABI with pinned host buffers (geometry
                     upload, BVH build, material upload, solve, flux download every
                     step).
  --impl reference   the reference algorithm on the host cores (the CPU oracle,
                     OpenMP, all threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rays/s and solves/s (batched/served vs plain, 1 GB300) at <=1e-4 flux err; p50/p99"
UNIT = "rays/s"
# Counters of the dominant kernel from ncu captures, valid only for the kernel sources they were
# taken on: the code of KERNEL_SOURCES (comments dropped) hashed to `sources`.  When the sources change, the bench reports the
# counters as stale (traffic null) until they are captured again.
#   traffic_per_launch: dram__bytes_read.sum + dram__bytes_write.sum of one diffuse launch on
#     this workload (1 M triangles, 3 bands, 450 M rays), mean of three captured launches;
#   the rest: one --set full capture of the same kernel on a 100 k-triangle orchard (45 M rays).
KERNEL_SOURCES = ["hrt_trace.cuh", "hrt_trace_w4.cuh", "hrt_device.cuh", "hrt_internal.h", "hrt_ps_w4.cu",
                  "hrt_ps_accumulate.cu", "hrt_bvh4.cu", "hrt_bvh.cu"]
PROFILE = {
    "sources": "2b1c1ad239ac",
    "kernel": "k_diffuse_w4<4,0,0,4,16,256,1,0,1> (lean4-s16; lean4-s32 is within 1 %)",
    "traffic_per_launch": 2.425e9,   # 2.371 GB read + 0.054 GB written, mean of 3 launches at 1 M
    "issue_active_pct": 83.5,
    "l1_hit_pct": 51.4,   # sector hit rate of 32-byte node loads (no second 16-byte load per sector)
    "l2_hit_pct": 92.9,
    "warps_active_pct": 49.8,
    "local_requests_per_ray": 0.232,  # (6.42 M + 4.02 M) / 45 M rays
    "top_stall": "not_selected 2.27, wait 2.11, long_scoreboard 1.65 per issued instruction",
}
ACC_DIRECT_RAYS, ACC_DIFFUSE_RAYS = 4, 9  # the accuracy leg's reduced ray counts
# diffuse-trace variants by the tuner's names (hrt_set_tuning(16 + v) forces one)
VARIANTS = {"binary4": 1, "binary3": 2, "simple": 3, "wide4": 4, "wide4-3": 5, "lean4": 6, "lean5": 7,
            "lean4-s16": 8, "lean4-b128": 9, "lean4-b512": 10, "lean4-k4": 11, "lean4-k16": 12,
            "lean4-s32": 13}


def code_digest(paths):
    """Hash of source files' code: comments, blank lines and surrounding spaces are dropped
    first, so editing a comment does not change it."""
    import hashlib
    import re

    h = hashlib.sha256()
    for p in paths:
        with open(p, encoding="utf-8") as fh:
            text = re.sub(r"/\*.*?\*/", "", fh.read(), flags=re.S)
        for line in text.splitlines():
            code = re.sub(r"//.*$", "", line).strip()
            if code:
                h.update(code.encode() + b"\n")
    return h.hexdigest()[:12]


def kernel_sources_digest():
    return code_digest([os.path.join(ROOT, "helios_gb300", "csrc", f) for f in KERNEL_SOURCES])


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def orchard_model(nx=20, ny=10, device=0, **kw):
    from helios_gb300 import workloads

    return workloads.orchard_model(nx=nx, ny=ny, device=device, **kw)


BANDS = ["LW", "NIR", "PAR"]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, nm in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def cpu_sample(rad, seconds_hint=15.0, threads=0, prim_limit=None):
    """The CPU oracle (the reference algorithm restated, FP64, OpenMP) on the first
    prim_limit primitives of the same workload; returns (rays/s, cores, sample text, t)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle
    from helpers import oracle_solve

    oracle.build()
    T, ty, ts = rad.geometry_arrays()
    sc = oracle.OracleScene(T, ty, ts)
    desc = rad.solve_description(BANDS, seed=1)
    cores = threads or os.cpu_count()
    if prim_limit is None:
        # calibrate: a small sample, then scale to ~seconds_hint
        t0 = time.perf_counter()
        _, st = sc.run_band(oracle_solve(desc), threads=cores, prim_limit=200)
        dt = max(time.perf_counter() - t0, 1e-3)
        prim_limit = int(min(T.shape[0], max(200, 200 * seconds_hint / dt)))
    t0 = time.perf_counter()
    _, st = sc.run_band(oracle_solve(desc), threads=cores, prim_limit=prim_limit)
    dt = time.perf_counter() - t0
    return st["rays"] / dt, cores, prim_limit, dt, st


def accuracy_and_cpu(rad, ctx, desc, threads=0):
    """The CPU-baseline leg, which is also the accuracy check of the timed kernels: the CPU
    oracle (the reference algorithm restated, FP64, OpenMP on all host threads) solves the
    whole orchard -- every primitive, all three bands, depth 5 -- at reduced ray counts
    (ACC_DIRECT_RAYS direct, ACC_DIFFUSE_RAYS diffuse per primitive), timed as the CPU
    baseline; the GPU solves the same seeded ray set with the benchmark's kernels; the
    per-primitive flux error of the GPU against the oracle is reported per band."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle
    from helpers import oracle_solve
    from helios_gb300 import workloads

    oracle.build()
    red = dict(desc)
    red["direct_rays"] = np.full_like(np.asarray(desc["direct_rays"]), ACC_DIRECT_RAYS)
    red["diffuse_rays"] = np.full_like(np.asarray(desc["diffuse_rays"]), ACC_DIFFUSE_RAYS)
    gpu = np.asarray(ctx.run_band(red, out=True), np.float64).reshape(desc["n"], -1)
    gpu_rays = ctx.last_stats()["rays"]
    T, ty, ts = rad.geometry_arrays()
    sc = oracle.OracleScene(T, ty, ts)
    cores = threads or os.cpu_count()
    t0 = time.perf_counter()
    ref, st = sc.run_band(oracle_solve(red), threads=cores)
    dt = time.perf_counter() - t0
    errs = {b: workloads.max_rel_err(gpu[:, i], ref[:, i]) for i, b in enumerate(BANDS)}
    cpu = {"value": st["rays"] / dt, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"CPU oracle runBand over all {desc['n']} primitives, 3 bands, depth 5, at {ACC_DIRECT_RAYS} "
                     f"direct / {ACC_DIFFUSE_RAYS} diffuse rays per primitive ({st['rays']} rays, {dt:.1f} s)"}
    acc = {"max_rel_err": max(errs.values()), "per_band": errs, "primitives": int(desc["n"]),
           "rays": int(st["rays"]), "same_rays": bool(gpu_rays == st["rays"]),
           "against": "FP64 oracle on the same Philox ray set (values below 1e-3 x mean compared against that floor)",
           "ray_counts": f"{ACC_DIRECT_RAYS} direct / {ACC_DIFFUSE_RAYS} diffuse per primitive; the timed solve uses "
                         "100 / 225 with the same kernels"}
    return cpu, acc


def run_reference(args):
    rad, sc = orchard_model(nx=args.trees[0], ny=args.trees[1])
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    times, rays = [], 0
    plim = None
    for i in range(args.warmup + args.steps):
        rps, cores, plim, dt, st = cpu_sample(rad, seconds_hint=args.ref_seconds, prim_limit=plim)
        if i >= args.warmup:
            times.append(dt)
            rays += st["rays"]
    val = rays / sum(times)
    sample = (f"oracle runBand restricted to rays launched from the first {plim} of {sc.n} primitives "
              f"(all passes, all bands), {cores} threads")
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 geometry / f64 sums",
            "data": "synthetic (seeded)", "config": {"workload": f"orchard-{sc.n}-triangles-3band", "primitives": sc.n},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_batched(rad, ctx, desc, stream, args):
    """Day sweep: 96 sun positions x (PAR, NIR) = 192 solves of the same orchard in one
    graph-captured launch, against plain single-band runBand solves on the same GPU."""
    import torch

    from helios_gb300 import scenes

    dirs, direct, diffuse, _ = scenes.day_sweep(latitude_deg=38.5, day_of_year=180, n=96, bands=("NIR", "PAR"))
    bands_sorted = sorted(["LW", "NIR", "PAR"])
    cols = [bands_sorted.index("NIR"), bands_sorted.index("PAR")]
    rho = desc["rho"][0][:, cols]
    tau = desc["tau"][0][:, cols]
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.run_sweep(dirs, direct, diffuse, rho, tau, 100, 200, 5, seed=7, out=False)  # capture + warm-up
    torch.cuda.synchronize()
    ev0.record(stream)
    reps = max(1, min(args.steps, 2))
    for _ in range(reps):
        ctx.run_sweep(dirs, direct, diffuse, rho, tau, 100, 200, 5, seed=7, out=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_sweep = ev0.elapsed_time(ev1) / 1e3 / reps
    sweep_rays = ctx.last_stats()["rays"]
    # plain: one runBand per (sun, band); timed on single-band solves at the bench's sun
    plain = rad.solve_description(["PAR"])
    ctx.run_band(plain, out=False)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(2):
        ctx.run_band(plain, out=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_plain = ev0.elapsed_time(ev1) / 1e3 / 2
    plain_rays = ctx.last_stats()["rays"]
    nsol = dirs.shape[0] * 2
    return {"workload": "day sweep: 96 sun positions (15 min, 38.5N, day 180) x PAR, NIR = 192 solves, depth 5",
            "s_per_sweep": t_sweep, "solves_per_s": nsol / t_sweep, "rays_per_sweep": sweep_rays,
            "rays_per_s": sweep_rays / t_sweep, "plain_s_per_solve": t_plain, "plain_solves_per_s": 1.0 / t_plain,
            "plain_rays_per_solve": plain_rays, "speedup_solves_per_s": (nsol / t_sweep) * t_plain,
            "graph_kernels": ctx.last_stats()["kernels"],
            "autotune": [x for x in ctx.tuning_report().splitlines() if x.startswith("record")],
            "plain_note": "plain = one single-band runBand (direct + primary diffuse + 5 scattering passes) timed "
                          "twice; 192 plain solves take 192x that"}


def run_served(args, device=0):
    """Served stream: Poisson arrivals at 50/s of requests on homogeneous-canopy scenes
    with sizes log-uniform in [2k, 2M] (patch:triangle 1:1), LAI U[0.5, 5], per scene 1-4
    bands, 50-400 diffuse rays and a seed; per request a sun at zenith U[0,75]; 100 direct
    rays, scattering depth 1; through the continuous-batching server, against the plain
    per-solve path (geometry upload + BVH build + solve per request, one at a time) on the
    same requests."""
    from helios_gb300 import _hrt, scenes

    sizes, lais, reqs = scenes.served_stream(n_requests=args.serve_requests, rate=50.0, n_scenes=args.serve_scenes,
                                             seed=0)
    built = {}
    used = sorted({r["scene"] for r in reqs})
    for k in used:
        built[k] = scenes.mixed_canopy(int(sizes[k]), float(lais[k]), seed=k)

    def mats(sc):
        rho = np.tile(scenes.SERVED_RHO, (sc.n, 1))
        tau = np.tile(scenes.SERVED_TAU, (sc.n, 1))
        rho[0] = 0.0
        tau[0] = 0.0
        return rho, tau

    depth = 1
    srv = _hrt.Server(device=device, workers=32, hbm_budget=64 << 30)
    for k in used:
        rho, tau = mats(built[k])
        srv.add_scene(k, built[k].T, built[k].ptype, built[k].twosided, rho, tau)
    for r in reqs:
        srv.submit(r["id"], r["scene"], r["arrival"], r["bands"], r["sun"], r["direct"], r["diffuse"], 100,
                   r["diffuse_rays"], depth, r["seed"])
    t0 = time.perf_counter()
    srv.start()
    srv.wait()
    wall = time.perf_counter() - t0
    res = [srv.result(r["id"]) for r in reqs]
    lat = np.array([x["done"] - x["arrival"] for x in res])
    rays = sum(x["rays"] for x in res)
    span = max(x["done"] for x in res) - min(x["arrival"] for x in res)
    st = srv.stats()
    srv.close()
    # plain per-solve path on the same requests (a prefix when --serve-plain is smaller)
    nplain = min(len(reqs), args.serve_plain) if args.serve_plain > 0 else len(reqs)
    ctx = _hrt.Context(device)
    t0 = time.perf_counter()
    cur = None
    for r in reqs[:nplain]:
        sc = built[r["scene"]]
        rho, tau = mats(sc)
        bl = int(r["bands"].sum())
        if r["scene"] != cur:  # the plain path rebuilds only when the scene changes
            ctx.update_geometry(sc.T, sc.ptype, sc.twosided)
            ctx.build_accel()
            cur = r["scene"]
        ctx.run_band({"band_launch": r["bands"], "sources": [{"type": 0, "position": tuple(r["sun"])}],
                      "source_flux": r["direct"], "rho": rho, "tau": tau, "diffuse_flux": r["diffuse"],
                      "direct_rays": np.full(bl, 100), "diffuse_rays": np.full(bl, r["diffuse_rays"]),
                      "depth": np.full(bl, depth), "emission": np.zeros(bl, np.uint8), "seed": r["seed"]})
    t_plain = time.perf_counter() - t0
    served_sps = len(reqs) / span
    plain_sps = nplain / t_plain
    return {"workload": f"{len(reqs)} requests, Poisson 50/s, {len(used)} canopy scenes log-uniform 2k-2M "
                        f"(patch:triangle 1:1), LAI U[0.5,5], 1-4 bands, zenith U[0,75], 50-400 diffuse rays, "
                        f"100 direct, depth {depth}",
            "offered_rate_per_s": 50.0, "solves_per_s": served_sps, "rays_per_s": rays / span,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "wall_s": wall, "bvh_builds": st["builds"], "evictions": st["evictions"],
            "batches": st["batches"], "requests_per_batch": st["batched_requests"] / max(st["batches"], 1),
            "multi_scene_groups": st["groups"], "batches_in_groups": st["grouped_batches"],
            "plain_solves_per_s": plain_sps, "plain_requests_timed": nplain,
            "speedup_solves_per_s": served_sps / plain_sps}


def stress_model(scale=1.0, device=0):
    """Deep-scattering stress workload: 3 M equilateral 3 cm triangles, 0.5 M 4 cm square
    patches and 0.5 M disks of 2 cm radius (two-sided, spherical leaf angles, uniform in
    a 24 x 24 x 4 m periodic box) over a one-sided ground, plus a 64^3 voxel grid over
    the same box with leaf area density U[0, 2]; NIR (rho 0.45, tau 0.40 for leaves and
    voxels), sun at zenith 30 deg (400 W/m^2) and 100 W/m^2 sky, 100 direct and 400
    (20 x 20) diffuse rays, scattering depth 20 with the FP64 residual stop at 1e-6.
    `scale` shrinks the primitive counts (and the voxel grid by its cube root)."""
    from helios_gb300 import scenes
    from helios_gb300.radiation import Context, RadiationModel

    div = max(2, int(round(64 * scale ** (1.0 / 3.0))))
    sc = scenes.deep_scatter(n_tri=int(3_000_000 * scale), n_patch=int(500_000 * scale),
                             n_disk=int(500_000 * scale), vox_div=div, seed=0)
    ctx = Context()
    ctx.addScene(sc)
    n = sc.n
    leaves = np.arange(1, n)
    ctx.setPrimitiveData(leaves, "reflectivity_NIR", np.full(n - 1, 0.45))
    ctx.setPrimitiveData(leaves, "transmissivity_NIR", np.full(n - 1, 0.40))
    rad = RadiationModel(ctx, device=device)
    rad.enforcePeriodicBoundary("xy")
    rad.addRadiationBand("NIR")
    rad.disableEmission("NIR")
    rad.setDirectRayCount("NIR", 100)
    rad.setDiffuseRayCount("NIR", 400)
    rad.setDiffuseRadiationFlux("NIR", 100.0)
    rad.setScatteringDepth("NIR", 20)
    rad.setScatteringResidualTolerance(1e-6)
    sun = rad.addCollimatedRadiationSource(scenes.sun_direction(30.0, 0.0))
    rad.setSourceFlux(sun, "NIR", 400.0)
    return rad, sc


# kernel variants by the tuner's names (hrt_set_tuning: 16 + v forces variant v)
TUNER_VARIANTS = {"binary4": 1, "binary3": 2, "simple": 3, "wide4": 4, "wide4-3": 5}


def run_stress(args, stream, device=0):
    """One timed solve of the deep-scattering stress workload (after one untimed solve)."""
    import torch

    rad, sc = stress_model(args.stress_scale, device=device)
    rad.ctx.set_stream(stream.cuda_stream)
    rad.setSeed(99)
    t0 = time.perf_counter()
    rad.updateGeometry()
    t_build = time.perf_counter() - t0
    desc = rad.solve_description(["NIR"])
    ctx = rad.ctx
    ctx.run_band(desc, out=False)  # untimed: tuning, first touch
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    ctx.run_band(desc, out=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    t = ev0.elapsed_time(ev1) / 1e3
    st = ctx.last_stats()
    tuning = [x for x in ctx.tuning_report().splitlines() if x.startswith("accumulate")]
    # traversal counts (untimed) on the same workload scaled to 5 % of the primitives, with
    # the kernel variant and tree the tuner chose for the full workload
    small, _ = stress_model(0.05 * args.stress_scale, device=device)
    small.setSeed(99)
    small.updateGeometry()
    chosen = tuning[-1].rsplit("-> ", 1)[-1].strip() if tuning else ""
    if chosen in TUNER_VARIANTS:
        small.ctx.set_tuning(16 + TUNER_VARIANTS[chosen])
    small.ctx.set_measure(1)
    small.ctx.run_band(small.solve_description(["NIR"]), out=False)
    meas = small.ctx.get_measure()
    small_rays = max(small.ctx.last_stats()["rays"], 1)
    counts = np.bincount(sc.ptype, minlength=5)
    return {"workload": f"deep scatter: {int(counts[1])} triangles, {int(counts[0]) - 1} patches, "
                        f"{int(counts[2])} disks, {int(counts[4])} voxels (LAD U[0,2]) + ground, NIR, "
                        "100 direct / 400 diffuse rays, depth 20, FP64 residual stop 1e-6",
            "primitives": int(sc.n), "s_per_solve": t, "rays_per_solve": st["rays"], "rays_per_s": st["rays"] / t,
            "scattering_iterations": st["iterations"], "kernels": st["kernels"], "setup_build_s": t_build,
            "node_visits_per_ray_5pct": meas["node_visits"] / small_rays,
            "prim_tests_per_ray_5pct": meas["prim_tests"] / small_rays, "counted_variant": chosen,
            "autotune": tuning}


def run_gpu(args):
    import torch

    from helios_gb300 import _hrt

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    rad, sc = orchard_model(nx=args.trees[0], ny=args.trees[1], device=local)
    stream = torch.cuda.Stream(device=local)
    rad.ctx.set_stream(stream.cuda_stream)
    if args.variant:
        rad.ctx.set_tuning(16 + VARIANTS[args.variant])  # profiling: one kernel, no tuner trials
    rad.setSeed(1234 + rank)
    t_setup = time.perf_counter()
    rad.updateGeometry()
    desc = rad.solve_description(BANDS)
    ctx = rad.ctx
    # first solve uploads materials, sources, emissivity and temperature
    ctx.run_band(desc, out=False)
    resident = {k: desc[k] for k in ("band_launch", "source_flux", "diffuse_flux", "diffuse_ext", "diffuse_norm",
                                     "diffuse_peak", "prague", "direct_rays", "diffuse_rays", "depth",
                                     "emission", "seed")}
    resident["nsources"] = len(desc["sources"])
    setup_s = time.perf_counter() - t_setup
    for _ in range(args.warmup):
        ctx.run_band(resident, out=False)
    rays_per_step = ctx.last_stats()["rays"]
    # traversal statistics (untimed): node visits and primitive tests per ray
    ctx.set_measure(1)
    ctx.run_band(resident, out=False)
    stats = ctx.get_measure()
    ctx.set_measure(2)  # time each trace-kernel launch in the timed region
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            ctx.run_band(resident, out=False)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    kernels_per_step = int(ctx.last_stats()["kernels"])  # before other solves overwrite the statistics
    meas = ctx.get_measure()
    ctx.set_measure(0)
    ms_t = torch.tensor([ms], device=f"cuda:{local}")
    if world > 1:
        torch.distributed.all_reduce(ms_t, op=torch.distributed.ReduceOp.MAX)
    ms = float(ms_t.item())
    # end to end through the C ABI with host buffers in pinned memory: every step uploads the
    # geometry and the materials, builds the trees, solves and reads the fluxes back
    keep = []

    def pinned(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        keep.append(t)
        v = t.numpy().view(a.dtype).reshape(a.shape)
        v[...] = a
        return v

    T, ty, ts = (pinned(np.ascontiguousarray(a)) for a in rad.geometry_arrays())
    full = dict(desc)
    for k in ("rho", "tau", "eps", "temperature"):
        full[k] = pinned(np.ascontiguousarray(desc[k]))
    h2d = T.nbytes + ty.nbytes + ts.nbytes + sum(full[k].nbytes for k in ("rho", "tau", "eps", "temperature"))
    flux_out = pinned(np.zeros((sc.n, len(BANDS)), np.float32))
    d2h = flux_out.nbytes
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.update_geometry(T, ty, ts)
        ctx.build_accel()
        flux = ctx.run_band(full, out=True, flux_out=flux_out)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    batched = None
    if not args.no_batched:
        batched = run_batched(rad, ctx, desc, stream, args)
    served = None
    if args.serve_requests > 0:
        served = run_served(args, device=local)
    stress = {"measured": False,
              "why": "one solve of the 4 M-primitive + 64^3-voxel scene at depth 20 is ~72 G rays and takes minutes "
                     "on one GB300, beyond the default run; bench.py --stress times it"}
    if args.stress:
        stress = run_stress(args, stream, device=local)
    if rank != 0:
        return
    hbm, peak_kind = peaks()
    # algorithmic bytes of the diffuse kernel (dominant): per ray 64 B per node visit,
    # 48 B per primitive test, origin record 64 B, per-band gather 4 B on hits and 8 B accumulate;
    # per launch: the mean bytes per diffuse ray of the statistics solve (visits and tests of
    # its diffuse launches only) x the rays of one diffuse launch
    diffuse_rays = max(stats["diffuse_rays"], 1)
    bytes_per_ray = (64.0 * stats["diffuse_node_visits"] + 48.0 * stats["diffuse_prim_tests"]) / diffuse_rays \
        + (64 + 4 * 3)
    rays_per_launch = stats["diffuse_rays"] / max(stats["diffuse_launches"], 1)
    diff_ms = meas["diffuse_ms"] / max(meas["diffuse_launches"], 1)
    diff_share = meas["diffuse_ms"] / max(meas["diffuse_ms"] + meas["direct_ms"], 1e-9)
    bytes_per_launch = bytes_per_ray * rays_per_launch
    achieved = bytes_per_launch / (diff_ms * 1e-3) / 1e9
    # ncu counters of the dominant kernel: used only while the kernel sources are the ones
    # they were captured on, and the workload is the one they were captured for
    digest = kernel_sources_digest()
    fresh = PROFILE["sources"] == digest and sc.n == 1_000_000
    traffic = PROFILE["traffic_per_launch"] if fresh else None
    chosen = [x.rsplit("-> ", 1)[-1] for x in ctx.tuning_report().splitlines()
              if x.startswith("accumulate") and "bands=3" in x]
    rps = rays_per_step * world / (ms * 1e-3)
    cpu, accuracy = None, None
    if not args.no_cpu:
        cpu, accuracy = accuracy_and_cpu(rad, ctx, desc)
    line = {
        "metric": METRIC, "value": rps, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 geometry / f64 sums", "data": "synthetic (seeded, seed 0)",
        "config": {"workload": f"orchard-{sc.n}-triangles-3band", "primitives": sc.n, "bands": BANDS,
                   "direct_rays": 100, "diffuse_rays": 225, "scattering_depth": 5,
                   "rays_per_step": rays_per_step, "solves_per_s": 1e3 / ms * world,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "working set (BVH 64 MB + records 128 MB + buffers) larger than the 129 MB L2; no flush",
                   "setup_s": setup_s},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "kernel": "k_diffuse_w4" if chosen and chosen[0].startswith("lean") else "k_diffuse_ps",
                     "variant": chosen[0] if chosen else None,
                     "limiter": "SM issue and L1/L2 hit latency of the node fetches, not DRAM: the algorithmic "
                                "bytes are logical fetches, almost all served by L1/L2 (traffic = DRAM bytes)",
                     "ncu": dict(PROFILE, sources_now=digest, stale=not fresh),
                     "kernel_ms": diff_ms, "kernel_share": diff_share, "bytes_per_launch": bytes_per_launch,
                     "rays_per_launch": rays_per_launch,
                     "node_visits_per_ray": stats["node_visits"] / max(rays_per_step, 1),
                     "prim_tests_per_ray": stats["prim_tests"] / max(rays_per_step, 1),
                     "diffuse_node_visits_per_ray": stats["diffuse_node_visits"] / diffuse_rays,
                     "diffuse_prim_tests_per_ray": stats["diffuse_prim_tests"] / diffuse_rays},
        "autotune": [x for x in ctx.tuning_report().splitlines() if x.startswith("accumulate")],
        "clocks": clk.summary(),
        "e2e": {"value": rays_per_step / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "s_per_step": e2e_s},
        "gpu_launches": None,
        "cpu_baseline": cpu,
        "accuracy": accuracy,
        "batched": batched,
        "served": served,
        "stress": stress,
    }
    line["gpu_launches"] = kernels_per_step * args.steps
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="hrt", choices=["hrt", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the day-sweep measurement")
    ap.add_argument("--serve-requests", type=int, default=2000, help="served-stream requests (0 = skip)")
    ap.add_argument("--serve-scenes", type=int, default=16, help="distinct scenes in the served stream")
    ap.add_argument("--serve-plain", type=int, default=200,
                    help="requests timed on the plain per-solve path (0 = all of them)")
    ap.add_argument("--ref-seconds", type=float, default=15.0)
    ap.add_argument("--trees", type=int, nargs=2, default=(20, 10), help="orchard grid (default 20 x 10 = 1M leaves)")
    ap.add_argument("--stress", action="store_true", help="also time the deep-scattering stress workload")
    ap.add_argument("--variant", choices=sorted(VARIANTS), default=None,
                    help="force one diffuse-trace variant instead of tuning (for profiling captures)")
    ap.add_argument("--stress-scale", type=float, default=1.0, help="primitive-count scale of the stress workload")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
