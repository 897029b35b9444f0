"""ctypes front end of the CPU FP64 oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` (as the checker) and bench.py's CPU
baseline legs import this module.  The product path never does.

The oracle restates the reference's radiation solve (PlantSimulationLab/Helios,
``plugins/radiation``): ray generation and energy deposition of
``src/optix8/OptiX8DeviceCode.cu`` and the pass orchestration of
``RadiationModel::runBand`` (``src/RadiationModel.cpp:3470-4663``).  See
``hrt_oracle.cpp`` for line-level citations.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libhrt_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library with its Makefile (gcc, OpenMP)."""
    src = os.path.join(_HERE, "hrt_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _Geometry(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("T", C.c_void_p),
        ("type", C.c_void_p),
        ("twosided", C.c_void_p),
        ("nbbox", C.c_int32),
        ("bbox_verts", C.c_void_p),
        ("periodic_x", C.c_float),
        ("periodic_y", C.c_float),
        ("voxel_lad", C.c_void_p),
        ("mask_id", C.c_void_p),
        ("uv_id", C.c_void_p),
        ("uv", C.c_void_p),
        ("nmasks", C.c_int32),
        ("mask_size", C.c_void_p),
        ("mask_data", C.c_void_p),
    ]


class _Solve(C.Structure):
    _fields_ = [
        ("nbands_global", C.c_int32),
        ("band_launch", C.c_void_p),
        ("nsources", C.c_int32),
        ("source_type", C.c_void_p),
        ("source_pos", C.c_void_p),
        ("source_width", C.c_void_p),
        ("source_rot", C.c_void_p),
        ("source_flux", C.c_void_p),
        ("rho", C.c_void_p),
        ("tau", C.c_void_p),
        ("diffuse_flux", C.c_void_p),
        ("diffuse_ext", C.c_void_p),
        ("diffuse_norm", C.c_void_p),
        ("diffuse_peak", C.c_void_p),
        ("prague", C.c_void_p),
        ("direct_rays", C.c_void_p),
        ("diffuse_rays", C.c_void_p),
        ("depth", C.c_void_p),
        ("emission", C.c_void_p),
        ("eps", C.c_void_p),
        ("temperature", C.c_void_p),
        ("seed", C.c_uint32),
        ("threads", C.c_int32),
        ("prim_limit", C.c_int32),
        ("scatter_tol", C.c_double),
        ("glass_nsrc", C.c_int32),
        ("is_glass", C.c_void_p),
        ("glass_n", C.c_void_p),
        ("glass_kl", C.c_void_p),
        ("ncameras", C.c_int32),
        ("cameras", C.c_void_p),
        ("cam_sky_radiance", C.c_void_p),
        ("cam_disk_radiance", C.c_void_p),
        ("cam_diffuse_flux", C.c_void_p),
        ("cam_prague", C.c_void_p),
        ("cam_emission", C.c_void_p),
        ("cam_sun", C.c_float * 3),
        ("cam_disk_cos", C.c_float),
    ]


class _Camera(C.Structure):
    _fields_ = [
        ("position", C.c_float * 3),
        ("direction", C.c_float * 2),
        ("focal_length", C.c_float),
        ("lens_diameter", C.c_float),
        ("fov_aspect", C.c_float),
        ("viewplane_length", C.c_float),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("antialiasing", C.c_int32),
        ("seed", C.c_uint32),
        ("camera_id", C.c_uint32),
        ("pixels", C.c_void_p),
        ("labels", C.c_void_p),
        ("depths", C.c_void_p),
    ]


def _load():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.orc_scene_create.restype = C.c_void_p
        _lib.orc_scene_create.argtypes = [C.POINTER(_Geometry)]
        _lib.orc_scene_destroy.argtypes = [C.c_void_p]
        _lib.orc_scene_bvh.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_trace.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_float, C.c_float,
                                   C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        _lib.orc_gen_rays.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.c_uint32, C.c_int32, C.c_int32,
                                      C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_run_band.argtypes = [C.c_void_p, C.POINTER(_Solve), C.c_void_p, C.c_void_p]
        _lib.orc_philox.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_set_rng.argtypes = [C.c_int]
        _lib.orc_sincos2pi.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_ln_unit.argtypes = [C.c_int64, C.c_void_p, C.c_void_p]
        _lib.orc_glass_trs.argtypes = [C.c_int64, C.c_void_p, C.c_float, C.c_float, C.c_void_p]
        _lib.orc_energy_balance.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float,
                                            C.c_void_p, C.c_void_p]
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


class OracleScene:
    """Host scene: primitive records, the host LBVH twin and the FP64 solver."""

    def __init__(self, T, ptype, twosided, bbox_verts=None, periodic=(0.0, 0.0), voxel_lad=None, masks=None):
        """masks: None or dict(mask_id [n] int, uv_id [n] int or None, uv [n, 8] or None,
        sizes [m, 2] (width, height), data: concatenated row-major uint8 masks)."""
        lib = _load()
        self.T = np.ascontiguousarray(T, dtype=np.float32).reshape(-1, 16)
        self.n = self.T.shape[0]
        self.type = np.ascontiguousarray(ptype, dtype=np.uint32)
        self.twosided = np.ascontiguousarray(twosided, dtype=np.int8)
        self.bbox = None if bbox_verts is None else np.ascontiguousarray(bbox_verts, dtype=np.float32)
        self.lad = None if voxel_lad is None else np.ascontiguousarray(voxel_lad, dtype=np.float32)
        g = _Geometry(self.n, _ptr(self.T), _ptr(self.type), _ptr(self.twosided),
                      0 if self.bbox is None else self.bbox.shape[0], _ptr(self.bbox),
                      float(periodic[0]), float(periodic[1]), _ptr(self.lad))
        self._mask_keep = []
        if masks is not None:
            mid = np.ascontiguousarray(masks["mask_id"], np.int32)
            sizes = np.ascontiguousarray(masks["sizes"], np.int32).reshape(-1, 2)
            data = np.ascontiguousarray(masks["data"], np.uint8)
            uvid = None if masks.get("uv_id") is None else np.ascontiguousarray(masks["uv_id"], np.int32)
            uv = None if masks.get("uv") is None else np.ascontiguousarray(masks["uv"], np.float32).reshape(-1, 8)
            self._mask_keep = [mid, sizes, data, uvid, uv]
            g.mask_id, g.uv_id, g.uv = _ptr(mid), _ptr(uvid), _ptr(uv)
            g.nmasks, g.mask_size, g.mask_data = sizes.shape[0], _ptr(sizes), _ptr(data)
        self._h = lib.orc_scene_create(C.byref(g))
        if not self._h:
            raise ValueError("oracle scene rejected (voxels need voxel_lad)")

    def close(self):
        if self._h:
            _load().orc_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bvh(self):
        n = self.n
        codes = np.zeros(n, np.uint64)
        perm = np.zeros(n, np.uint32)
        nodes = np.zeros((max(n - 1, 1), 16), np.uint32)
        _load().orc_scene_bvh(self._h, _ptr(codes), _ptr(perm), _ptr(nodes))
        return codes, perm, nodes

    def trace(self, o, d, mode=0, tmin=1e-4, tmax=1e38, threads=0):
        """mode 0: BVH closest hit; 1: brute force; 2: brute force, reference formulas; 3: BVH any hit."""
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        nr = o.shape[0]
        hit = np.zeros(nr, np.int32)
        t = np.zeros(nr, np.float32)
        face = np.zeros(nr, np.int32)
        cnt = np.zeros(2, np.uint64)
        _load().orc_trace(self._h, nr, _ptr(o), _ptr(d), tmin, tmax, mode, _ptr(hit), _ptr(t), _ptr(face),
                          _ptr(cnt), threads)
        return hit, t, face, cnt

    def gen_rays(self, kind, seed, pass_id, rpp, face=1, direction=(0.0, 0.0, 1.0)):
        dimx = max(int(np.sqrt(np.float32(rpp))), 1)
        nr = dimx * (rpp // dimx)
        o = np.zeros((self.n * nr, 3), np.float32)
        d = np.zeros((self.n * nr, 3), np.float32)
        dir3 = np.asarray(direction, np.float32)
        _load().orc_gen_rays(self._h, kind, seed, pass_id, rpp, face, _ptr(dir3), _ptr(o), _ptr(d))
        return o, d

    def run_band(self, solve: dict, threads=0, prim_limit=0):
        """Solve one runBand call; returns (flux [n, Bl] float64, stats dict)."""
        keep = []

        def arr(key, dtype, default=None):
            v = solve.get(key, default)
            if v is None:
                return None
            a = np.ascontiguousarray(v, dtype=dtype)
            keep.append(a)
            return a

        band_launch = arr("band_launch", np.uint8)
        bl = int(band_launch.sum())
        s = _Solve()
        s.nbands_global = band_launch.shape[0]
        s.band_launch = _ptr(band_launch)
        src_type = arr("source_type", np.int32)
        s.nsources = 0 if src_type is None else src_type.shape[0]
        s.source_type = _ptr(src_type)
        s.source_pos = _ptr(arr("source_pos", np.float32))
        s.source_width = _ptr(arr("source_width", np.float32))
        s.source_rot = _ptr(arr("source_rot", np.float32))
        s.source_flux = _ptr(arr("source_flux", np.float32))
        s.rho = _ptr(arr("rho", np.float32))
        s.tau = _ptr(arr("tau", np.float32))
        s.diffuse_flux = _ptr(arr("diffuse_flux", np.float32))
        s.diffuse_ext = _ptr(arr("diffuse_ext", np.float32))
        s.diffuse_norm = _ptr(arr("diffuse_norm", np.float32))
        s.diffuse_peak = _ptr(arr("diffuse_peak", np.float32))
        s.prague = _ptr(arr("prague", np.float32))
        s.direct_rays = _ptr(arr("direct_rays", np.int32))
        s.diffuse_rays = _ptr(arr("diffuse_rays", np.int32))
        s.depth = _ptr(arr("depth", np.int32))
        s.emission = _ptr(arr("emission", np.uint8))
        s.eps = _ptr(arr("eps", np.float32))
        s.temperature = _ptr(arr("temperature", np.float32))
        s.seed = int(solve.get("seed", 0)) & 0xFFFFFFFF
        s.threads = int(threads)
        s.prim_limit = int(prim_limit)
        s.scatter_tol = float(solve.get("scatter_tolerance", 0.0))
        ig = arr("is_glass", np.int8)
        if ig is not None:
            s.glass_nsrc = ig.shape[0]
            s.is_glass = _ptr(ig)
            s.glass_n = _ptr(arr("glass_n", np.float32))
            s.glass_kl = _ptr(arr("glass_kl", np.float32))
        cams = solve.get("cameras") or []
        cam_out = []
        if cams:
            arr = (_Camera * len(cams))()
            for i, cam in enumerate(cams):
                c = arr[i]
                for k in range(3):
                    c.position[k] = float(cam["position"][k])
                c.direction[0], c.direction[1] = float(cam["direction"][0]), float(cam["direction"][1])
                c.focal_length = float(cam["focal_length"])
                c.lens_diameter = float(cam["lens_diameter"])
                c.fov_aspect = float(cam["fov_aspect"])
                c.viewplane_length = float(cam["viewplane_length"])
                W, H = int(cam["resolution"][0]), int(cam["resolution"][1])
                c.width, c.height = W, H
                c.antialiasing = int(cam.get("antialiasing", 1))
                c.seed = int(cam.get("seed", 0)) & 0xFFFFFFFF
                c.camera_id = int(cam.get("camera_id", 0))
                out = {"pixels": np.zeros((H, W, bl), np.float32), "labels": np.zeros((H, W), np.uint32),
                       "depths": np.zeros((H, W), np.float32)}
                c.pixels, c.labels, c.depths = _ptr(out["pixels"]), _ptr(out["labels"]), _ptr(out["depths"])
                cam_out.append(out)
            keep.append(arr)
            s.ncameras = len(cams)
            s.cameras = C.cast(arr, C.c_void_p)
            sky = solve.get("camera_sky")
            if sky is not None:
                def sk(key, dtype):
                    v = sky.get(key)
                    if v is None:
                        return None
                    a = np.ascontiguousarray(v, dtype).ravel()
                    keep.append(a)
                    return _ptr(a)
                s.cam_sky_radiance = sk("sky_radiance", np.float32)
                s.cam_disk_radiance = sk("disk_radiance", np.float32)
                s.cam_diffuse_flux = sk("diffuse_flux", np.float32)
                s.cam_prague = sk("prague", np.float32)
                s.cam_emission = sk("emission", np.uint32)
                sun = sky.get("sun", (0.0, 0.0, 1.0))
                for k in range(3):
                    s.cam_sun[k] = float(sun[k])
                s.cam_disk_cos = float(sky.get("disk_cos", 0.0))
        flux = np.zeros((self.n, bl), np.float64)
        stats = np.zeros(5, np.uint64)
        _load().orc_run_band(self._h, C.byref(s), _ptr(flux), _ptr(stats))
        st = {"rays": int(stats[0]), "nodes": int(stats[1]), "prims": int(stats[2]),
              "hits": int(stats[3]), "iterations": int(stats[4])}
        if cams:
            st["cameras"] = cam_out
        return flux, st


class reference_rng:
    """Context manager: the ray generators draw from the reference's random-number stream
    (TEA-16 seeded 24-bit LCG per ray, OptiX8DeviceCode.cu:29-49) instead of Philox.  Results
    then agree with the product only in distribution (statistical parity)."""

    def __enter__(self):
        if _load().orc_set_rng(1):
            raise RuntimeError("orc_set_rng failed")
        return self

    def __exit__(self, *exc):
        _load().orc_set_rng(0)
        return False


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    _load().orc_philox(_ptr(c), _ptr(k), _ptr(out))
    return out


def sincos2pi(u):
    u = np.ascontiguousarray(u, np.float32)
    c = np.zeros_like(u)
    s = np.zeros_like(u)
    _load().orc_sincos2pi(u.size, _ptr(u), _ptr(c), _ptr(s))
    return c, s


def ln_unit(x):
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(x)
    _load().orc_ln_unit(x.size, _ptr(x), _ptr(out))
    return out


def glass_trs(cos_theta, n, kl):
    """(tau, rho, alpha) [m, 3] of one translucent sheet at the given incidence cosines."""
    c = np.ascontiguousarray(cos_theta, np.float32).ravel()
    out = np.zeros((c.size, 3), np.float32)
    _load().orc_glass_trs(c.size, _ptr(c), float(n), float(kl), _ptr(out))
    return out


EB_FIELDS = ("air_temperature", "air_vapor_pressure", "air_pressure", "bl_conductance", "moisture_conductance",
             "emissivity", "other_flux", "heat_capacity", "surface_humidity", "stomatal_sidedness")


def energy_balance(surf, net_radiation, temperature):
    """(T [n], fluxes [n, 5], unconverged) of the surface energy balance on the CPU (FP32)."""
    n = int(np.asarray(net_radiation).size)
    rows = [np.ascontiguousarray(surf[k], np.float32).ravel() for k in EB_FIELDS]
    rows.append(np.ascontiguousarray(net_radiation, np.float32).ravel())
    inp = np.ascontiguousarray(np.concatenate(rows), np.float32)
    ns = np.ascontiguousarray(surf["nsides"], np.uint8).ravel()
    Tin = np.ascontiguousarray(temperature, np.float32).ravel()
    T = np.zeros(n, np.float32)
    out = np.zeros((n, 5), np.float32)
    bad = _load().orc_energy_balance(n, _ptr(inp), _ptr(ns), _ptr(Tin), float(surf.get("dt", 0.0)),
                                     float(surf.get("temperature_default", 300.0)), _ptr(T), _ptr(out))
    return T, out, int(bad)
