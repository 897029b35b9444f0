"""ctypes binding of libhrt's C ABI (include/hrt.h).

The library is the product: there is no CPU fallback.  ``load()`` raises if
the shared object is missing, and every call that returns a non-zero code
raises ``HrtError`` with the context's error text.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhrt.so")

HRT_OK, HRT_EINVAL, HRT_ECUDA, HRT_ENOMEM, HRT_EDEVICE, HRT_EUNSUPPORTED = 0, -1, -2, -3, -4, -5

# Every function the header declares; the CPU test suite checks they are exported.
EXPORTS = [
    "hrt_create", "hrt_destroy", "hrt_last_error", "hrt_set_stream", "hrt_update_geometry", "hrt_build_accel",
    "hrt_update_materials", "hrt_update_sources", "hrt_upload_source_fluxes", "hrt_launch_direct",
    "hrt_launch_diffuse", "hrt_get_results", "hrt_zero_radiation_buffers", "hrt_zero_scatter_buffers",
    "hrt_copy_scatter_to_radiation", "hrt_upload_radiation_out", "hrt_query_memory", "hrt_backend_name",
    "hrt_run_band", "hrt_last_stats", "hrt_device_status", "hrt_trace_rays", "hrt_gen_rays", "hrt_get_bvh",
    "hrt_source_rotation", "hrt_set_measure", "hrt_get_measure", "hrt_build_accel_static", "hrt_run_sweep",
    "hrt_server_create", "hrt_server_add_scene", "hrt_server_submit", "hrt_server_start", "hrt_server_wait",
    "hrt_server_result", "hrt_server_stats", "hrt_server_destroy", "hrt_set_tuning", "hrt_tuning_report",
    "hrt_set_ray_budget", "hrt_update_glass", "hrt_update_sky_model", "hrt_launch_camera",
    "hrt_launch_pixel_labels", "hrt_zero_camera_pixel_buffers", "hrt_get_camera_results",
    "hrt_energy_balance", "hrt_run_coupled", "hrt_scene_load", "hrt_scene_last_error", "hrt_scene_count",
    "hrt_scene_arrays", "hrt_scene_data_labels", "hrt_scene_data", "hrt_scene_free",
    "hrt_plan_launch_chunks", "hrt_set_launch_ray_limit", "hrt_set_visit_budget", "hrt_run_sweep_multi",
]


def plan_launch_chunks(count: int, rays_per_primitive: int, max_rays: int = 0):
    """(launches, primitives per launch) for a pass (hrt_plan_launch_chunks; host arithmetic only).

    Raises HrtError(HRT_EUNSUPPORTED) when one primitive's rays exceed a launch."""
    lib = load()
    per = C.c_uint32()
    k = lib.hrt_plan_launch_chunks(int(count), int(rays_per_primitive), int(max_rays), C.byref(per))
    if k < 0:
        raise HrtError(int(k), "the rays of one primitive exceed the rays one launch can carry")
    return int(k), int(per.value)


class HrtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"hrt error {code}: {msg}")
        self.code = code


class Geometry(C.Structure):
    _fields_ = [("n", C.c_int32), ("transform", C.c_void_p), ("type", C.c_void_p), ("twosided", C.c_void_p),
                ("nbbox", C.c_int32), ("bbox_vertices", C.c_void_p), ("periodic_x", C.c_float),
                ("periodic_y", C.c_float), ("voxel_lad", C.c_void_p), ("mask_id", C.c_void_p),
                ("uv_id", C.c_void_p), ("uv", C.c_void_p), ("nmasks", C.c_int32), ("mask_size", C.c_void_p),
                ("mask_data", C.c_void_p)]


class Source(C.Structure):
    _fields_ = [("type", C.c_uint32), ("position", C.c_float * 3), ("width", C.c_float * 2),
                ("rotation", C.c_float * 3)]


class Launch(C.Structure):
    _fields_ = [("launch_offset", C.c_uint32), ("launch_count", C.c_uint32), ("rays_per_primitive", C.c_uint32),
                ("random_seed", C.c_uint32), ("pass_id", C.c_uint32), ("nbands_global", C.c_uint32),
                ("nbands_launch", C.c_uint32), ("band_launch_flag", C.c_void_p), ("launch_face", C.c_uint32),
                ("diffuse_flux", C.c_void_p), ("diffuse_extinction", C.c_void_p), ("diffuse_peak_dir", C.c_void_p),
                ("diffuse_dist_norm", C.c_void_p), ("sky_radiance_params", C.c_void_p),
                ("radiation_out_top", C.c_void_p), ("radiation_out_bottom", C.c_void_p)]


class BandSolve(C.Structure):
    _fields_ = [("nbands_global", C.c_int32), ("band_launch", C.c_void_p), ("nsources", C.c_int32),
                ("sources", C.c_void_p), ("source_flux", C.c_void_p), ("rho", C.c_void_p), ("tau", C.c_void_p),
                ("diffuse_flux", C.c_void_p), ("diffuse_extinction", C.c_void_p), ("diffuse_peak_dir", C.c_void_p),
                ("diffuse_dist_norm", C.c_void_p), ("sky_radiance_params", C.c_void_p),
                ("direct_rays", C.c_void_p), ("diffuse_rays", C.c_void_p), ("scattering_depth", C.c_void_p),
                ("emission", C.c_void_p), ("emissivity", C.c_void_p), ("temperature", C.c_void_p),
                ("seed", C.c_uint32), ("scatter_tolerance", C.c_double), ("ncameras", C.c_int32),
                ("cameras", C.c_void_p), ("camera_sky", C.c_void_p)]


class Surface(C.Structure):
    _fields_ = [("air_temperature", C.c_void_p), ("air_vapor_pressure", C.c_void_p), ("air_pressure", C.c_void_p),
                ("bl_conductance", C.c_void_p), ("moisture_conductance", C.c_void_p), ("emissivity", C.c_void_p),
                ("other_flux", C.c_void_p), ("heat_capacity", C.c_void_p), ("surface_humidity", C.c_void_p),
                ("stomatal_sidedness", C.c_void_p), ("nsides", C.c_void_p), ("dt", C.c_float),
                ("temperature_default", C.c_float)]


SURFACE_FIELDS = ("air_temperature", "air_vapor_pressure", "air_pressure", "bl_conductance", "moisture_conductance",
                  "emissivity", "other_flux", "heat_capacity", "surface_humidity", "stomatal_sidedness")


def make_surface(surf: dict, keep: list) -> Surface:
    """hrt_surface from a dict of [n] arrays (SURFACE_FIELDS, nsides) plus dt and temperature_default."""
    s = Surface()
    for k in SURFACE_FIELDS:
        a = np.ascontiguousarray(surf[k], np.float32).ravel()
        keep.append(a)
        setattr(s, k, ptr(a))
    ns = np.ascontiguousarray(surf["nsides"], np.uint8).ravel()
    keep.append(ns)
    s.nsides = ptr(ns)
    s.dt = float(surf.get("dt", 0.0))
    s.temperature_default = float(surf.get("temperature_default", 300.0))
    return s


class LoadOptions(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("height", C.c_float), ("rotation", C.c_float * 2),
                ("up_axis", C.c_int32), ("default_color", C.c_float * 3)]


UP_AXES = {"XUP": 0, "YUP": 1, "ZUP": 2}


def load_scene_file(path, origin=(0.0, 0.0, 0.0), height=0.0, rotation=(0.0, 0.0), up_axis="ZUP",
                    default_color=(0.0, 0.0, 1.0)):
    """Primitive arrays of a PLY / OBJ / XML file (hrt_scene_load): dict with T [n, 16], type [n],
    twosided [n], color [n, 3] and data {label: [n] float64 (NaN where absent)}."""
    lib = load()
    if up_axis not in UP_AXES:
        raise ValueError(f"{up_axis} is not a valid up-axis. Please specify a value of XUP, YUP, or ZUP.")
    o = LoadOptions()
    for k in range(3):
        o.origin[k] = float(origin[k])
        o.default_color[k] = float(default_color[k])
    o.height = float(height)
    o.rotation[0], o.rotation[1] = float(rotation[0]), float(rotation[1])
    o.up_axis = UP_AXES[up_axis]
    h = C.c_void_p()
    rc = lib.hrt_scene_load(os.fsencode(path), C.byref(o), C.byref(h))
    if rc != HRT_OK:
        raise HrtError(rc, lib.hrt_scene_last_error().decode())
    try:
        n = int(lib.hrt_scene_count(h))
        T = np.zeros((n, 16), np.float32)
        ty = np.zeros(n, np.uint32)
        ts = np.zeros(n, np.int8)
        col = np.zeros((n, 3), np.float32)
        lib.hrt_scene_arrays(h, ptr(T), ptr(ty), ptr(ts), ptr(col))
        need = lib.hrt_scene_data_labels(h, None, 0)
        buf = C.create_string_buffer(int(need))
        lib.hrt_scene_data_labels(h, buf, need)
        data = {}
        for lab in buf.value.decode().split("\n"):
            if lab:
                v = np.zeros(n, np.float64)
                lib.hrt_scene_data(h, lab.encode(), ptr(v))
                data[lab] = v
    finally:
        lib.hrt_scene_free(h)
    return {"T": T, "type": ty, "twosided": ts, "color": col, "data": data}


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("direction", C.c_float * 2), ("focal_length", C.c_float),
                ("lens_diameter", C.c_float), ("fov_aspect", C.c_float), ("viewplane_length", C.c_float),
                ("resolution", C.c_int32 * 2), ("tile_offset", C.c_int32 * 2), ("tile_resolution", C.c_int32 * 2),
                ("antialiasing", C.c_int32), ("seed", C.c_uint32), ("camera_id", C.c_uint32),
                ("pixels", C.c_void_p), ("labels", C.c_void_p), ("depths", C.c_void_p)]


class SkyModel(C.Structure):
    _fields_ = [("sky_radiance_params", C.c_void_p), ("camera_sky_radiance", C.c_void_p),
                ("sun_direction", C.c_float * 3), ("solar_disk_radiance", C.c_void_p),
                ("solar_disk_cos_angle", C.c_float), ("camera_diffuse_flux", C.c_void_p),
                ("band_emission_flag", C.c_void_p)]


def make_camera(cam: dict) -> Camera:
    """hrt_camera from a camera dict (the form the oracle takes)."""
    c = Camera()
    for k in range(3):
        c.position[k] = float(cam["position"][k])
    c.direction[0], c.direction[1] = float(cam["direction"][0]), float(cam["direction"][1])
    c.focal_length = float(cam["focal_length"])
    c.lens_diameter = float(cam["lens_diameter"])
    c.fov_aspect = float(cam["fov_aspect"])
    c.viewplane_length = float(cam["viewplane_length"])
    c.resolution[0], c.resolution[1] = int(cam["resolution"][0]), int(cam["resolution"][1])
    off = cam.get("tile_offset", (0, 0))
    tr = cam.get("tile_resolution", (0, 0))
    c.tile_offset[0], c.tile_offset[1] = int(off[0]), int(off[1])
    c.tile_resolution[0], c.tile_resolution[1] = int(tr[0]), int(tr[1])
    c.antialiasing = int(cam.get("antialiasing", 1))
    c.seed = int(cam.get("seed", 0)) & 0xFFFFFFFF
    c.camera_id = int(cam.get("camera_id", 0))
    return c


def make_sky_model(sky: dict, keep: list) -> SkyModel:
    """hrt_sky_model from a camera-sky dict; arrays referenced are appended to keep."""
    m = SkyModel()

    def a(key, dt):
        v = sky.get(key)
        if v is None:
            return None
        arr = np.ascontiguousarray(v, dt).ravel()
        keep.append(arr)
        return ptr(arr)

    m.sky_radiance_params = a("prague", np.float32)
    m.camera_sky_radiance = a("sky_radiance", np.float32)
    sun = sky.get("sun", (0.0, 0.0, 1.0))
    for k in range(3):
        m.sun_direction[k] = float(sun[k])
    m.solar_disk_radiance = a("disk_radiance", np.float32)
    m.solar_disk_cos_angle = float(sky.get("disk_cos", 0.0))
    m.camera_diffuse_flux = a("diffuse_flux", np.float32)
    m.band_emission_flag = a("emission", np.uint32)
    return m


class Sweep(C.Structure):
    _fields_ = [("nsun", C.c_int32), ("sun_dir", C.c_void_p), ("nbands", C.c_int32), ("direct_flux", C.c_void_p),
                ("diffuse_flux", C.c_void_p), ("rho", C.c_void_p), ("tau", C.c_void_p), ("direct_rays", C.c_int32),
                ("diffuse_rays", C.c_int32), ("scattering_depth", C.c_int32), ("seed", C.c_uint32)]


class ServeRequest(C.Structure):
    _fields_ = [("request_id", C.c_uint64), ("scene_id", C.c_uint32), ("arrival_s", C.c_double),
                ("band_launch", C.c_void_p), ("sun_dir", C.c_float * 3), ("source_flux", C.c_void_p),
                ("diffuse_flux", C.c_void_p), ("direct_rays", C.c_int32), ("diffuse_rays", C.c_int32),
                ("scattering_depth", C.c_int32), ("seed", C.c_uint32), ("keep_result", C.c_int32)]


_lib = None
VP = C.c_void_p


def load(path: str | None = None):
    """Load libhrt.so (build it first with helios_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"libhrt.so not found at {p}; run helios_gb300.build.build() (nvcc, sm_103a)")
    lib = C.CDLL(p)
    sig = {
        "hrt_create": (C.c_int, [C.POINTER(VP), C.c_int]),
        "hrt_destroy": (C.c_int, [VP]),
        "hrt_last_error": (C.c_char_p, [VP]),
        "hrt_set_stream": (C.c_int, [VP, VP]),
        "hrt_update_geometry": (C.c_int, [VP, C.POINTER(Geometry)]),
        "hrt_build_accel": (C.c_int, [VP]),
        "hrt_update_materials": (C.c_int, [VP, C.c_int32, C.c_int32, C.c_int32, VP, VP]),
        "hrt_update_glass": (C.c_int, [VP, C.c_int32, C.c_int32, C.c_int32, VP, VP, VP]),
        "hrt_update_sky_model": (C.c_int, [VP, C.c_int32, VP]),
        "hrt_launch_camera": (C.c_int, [VP, VP]),
        "hrt_launch_pixel_labels": (C.c_int, [VP, VP]),
        "hrt_zero_camera_pixel_buffers": (C.c_int, [VP, C.c_int32, C.c_int32]),
        "hrt_get_camera_results": (C.c_int, [VP, VP, VP, VP, C.c_int32, C.c_int32]),
        "hrt_energy_balance": (C.c_int, [VP, C.c_int32, VP, VP, VP, VP, VP]),
        "hrt_scene_load": (C.c_int, [C.c_char_p, VP, C.POINTER(C.c_void_p)]),
        "hrt_scene_last_error": (C.c_char_p, []),
        "hrt_scene_count": (C.c_int64, [VP]),
        "hrt_scene_arrays": (C.c_int, [VP, VP, VP, VP, VP]),
        "hrt_scene_data_labels": (C.c_size_t, [VP, VP, C.c_size_t]),
        "hrt_scene_data": (C.c_int, [VP, C.c_char_p, VP]),
        "hrt_scene_free": (None, [VP]),
        "hrt_run_coupled": (C.c_int, [VP, VP, VP, C.c_int32, C.c_float, VP, VP, VP]),
        "hrt_update_sources": (C.c_int, [VP, C.c_int32, VP]),
        "hrt_upload_source_fluxes": (C.c_int, [VP, VP, C.c_size_t]),
        "hrt_launch_direct": (C.c_int, [VP, C.POINTER(Launch)]),
        "hrt_launch_diffuse": (C.c_int, [VP, C.POINTER(Launch)]),
        "hrt_get_results": (C.c_int, [VP, VP, VP, VP, VP, VP]),
        "hrt_zero_radiation_buffers": (C.c_int, [VP, C.c_size_t]),
        "hrt_zero_scatter_buffers": (C.c_int, [VP]),
        "hrt_copy_scatter_to_radiation": (C.c_int, [VP]),
        "hrt_upload_radiation_out": (C.c_int, [VP, VP, VP, C.c_size_t]),
        "hrt_query_memory": (C.c_int, [VP, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
        "hrt_backend_name": (C.c_char_p, []),
        "hrt_run_band": (C.c_int, [VP, C.POINTER(BandSolve), VP]),
        "hrt_last_stats": (C.c_int, [VP, VP, C.c_int]),
        "hrt_set_tuning": (C.c_int, [VP, C.c_int]),
        "hrt_set_ray_budget": (C.c_int, [VP, C.c_uint32]),
        "hrt_plan_launch_chunks": (C.c_int64, [C.c_uint32, C.c_uint64, C.c_uint64, C.POINTER(C.c_uint32)]),
        "hrt_set_launch_ray_limit": (C.c_int, [VP, C.c_uint64]),
        "hrt_set_visit_budget": (C.c_int, [VP, C.c_uint32]),
        "hrt_tuning_report": (C.c_size_t, [VP, VP, C.c_size_t]),
        "hrt_device_status": (C.c_int, [VP, C.POINTER(C.c_uint32), C.c_int]),
        "hrt_trace_rays": (C.c_int, [VP, C.c_int64, VP, VP, C.c_float, C.c_float, C.c_int, VP, VP, VP]),
        "hrt_gen_rays": (C.c_int, [VP, C.c_int, C.c_uint32, C.c_uint32, C.c_int32, C.c_int32, VP, VP, VP]),
        "hrt_get_bvh": (C.c_int, [VP, VP, VP, VP]),
        "hrt_source_rotation": (None, [VP, VP]),
        "hrt_set_measure": (C.c_int, [VP, C.c_int]),
        "hrt_get_measure": (C.c_int, [VP, VP, C.c_int]),
        "hrt_build_accel_static": (C.c_int, [VP, VP, C.c_int32, VP, VP, VP, VP, VP, VP]),
        "hrt_run_sweep": (C.c_int, [VP, C.POINTER(Sweep), VP]),
        "hrt_run_sweep_multi": (C.c_int, [C.POINTER(VP), C.POINTER(Sweep), C.c_int32, C.POINTER(VP)]),
        "hrt_server_create": (C.c_int, [C.POINTER(VP), C.c_int, C.c_int, C.c_size_t]),
        "hrt_server_add_scene": (C.c_int, [VP, C.c_uint32, C.POINTER(Geometry), C.c_int32, VP, VP]),
        "hrt_server_submit": (C.c_int, [VP, C.POINTER(ServeRequest)]),
        "hrt_server_start": (C.c_int, [VP]),
        "hrt_server_wait": (C.c_int, [VP]),
        "hrt_server_result": (C.c_int, [VP, C.c_uint64, VP, C.c_size_t, VP, VP, VP]),
        "hrt_server_stats": (C.c_int, [VP, VP, C.c_int]),
        "hrt_server_destroy": (C.c_int, [VP]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def ptr(a):
    return None if a is None else a.ctypes.data


def f32(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(shape) if shape is not None else a


def source_rotation(rot) -> np.ndarray:
    r = np.ascontiguousarray(rot, np.float32)
    out = np.zeros(9, np.float32)
    load().hrt_source_rotation(ptr(r), ptr(out))
    return out


class Context:
    """An hrt_context: one device, one stream, device-resident scene and buffers."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.hrt_create(C.byref(h), device)
        if rc != HRT_OK:
            raise HrtError(rc, "hrt_create failed (no CUDA device?)")
        self.h = h
        self.n = 0
        self._keep = []

    def check(self, rc):
        if rc != HRT_OK:
            raise HrtError(rc, self.lib.hrt_last_error(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.hrt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None):
        self.check(self.lib.hrt_set_stream(self.h, stream_handle))

    # -------------------------------------------------------------- geometry
    def update_geometry(self, T, ptype, twosided, bbox_verts=None, periodic=(0.0, 0.0), voxel_lad=None,
                        masks=None):
        """voxel_lad: [n] leaf area density, read for voxel primitives (required when there are any).
        masks: None or dict(mask_id [n], uv_id [n] or None, uv [n, 8] or None, sizes [m, 2]
        (width, height), data: the masks' row-major uint8 texels one after another)."""
        T = f32(T).reshape(-1, 16)
        ty = np.ascontiguousarray(ptype, np.uint32)
        ts = np.ascontiguousarray(twosided, np.int8)
        bb = None if bbox_verts is None else f32(bbox_verts).reshape(-1, 4, 3)
        lad = None if voxel_lad is None else f32(voxel_lad)
        g = Geometry(T.shape[0], ptr(T), ptr(ty), ptr(ts), 0 if bb is None else bb.shape[0], ptr(bb),
                     float(periodic[0]), float(periodic[1]), ptr(lad))
        keep = []
        if masks is not None:
            mid = np.ascontiguousarray(masks["mask_id"], np.int32)
            sizes = np.ascontiguousarray(masks["sizes"], np.int32).reshape(-1, 2)
            data = np.ascontiguousarray(masks["data"], np.uint8)
            uvid = None if masks.get("uv_id") is None else np.ascontiguousarray(masks["uv_id"], np.int32)
            uv = None if masks.get("uv") is None else f32(masks["uv"]).reshape(-1, 8)
            keep = [mid, sizes, data, uvid, uv]
            g.mask_id, g.uv_id, g.uv = ptr(mid), ptr(uvid), ptr(uv)
            g.nmasks, g.mask_size, g.mask_data = sizes.shape[0], ptr(sizes), ptr(data)
        self.check(self.lib.hrt_update_geometry(self.h, C.byref(g)))
        del keep
        self.n = T.shape[0]

    def build_accel(self):
        self.check(self.lib.hrt_build_accel(self.h))

    def update_materials(self, rho, tau, nsources, nbands_global):
        rho, tau = f32(rho), f32(tau)
        self.check(self.lib.hrt_update_materials(self.h, nsources, self.n, nbands_global, ptr(rho), ptr(tau)))

    def update_glass(self, is_glass=None, glass_n=None, glass_kl=None):
        """Translucent covers [S, n, Bg] (is_glass None: none)."""
        if is_glass is None:
            self.check(self.lib.hrt_update_glass(self.h, 0, self.n, 0, None, None, None))
            return
        ig = np.ascontiguousarray(is_glass, np.int8)
        gn, gk = f32(glass_n), f32(glass_kl)
        S, n, Bg = ig.shape
        self.check(self.lib.hrt_update_glass(self.h, S, n, Bg, ptr(ig), ptr(gn), ptr(gk)))

    @staticmethod
    def make_sources(sources):
        arr = (Source * max(len(sources), 1))()
        for i, s in enumerate(sources):
            arr[i].type = int(s.get("type", 0))
            for k in range(3):
                arr[i].position[k] = float(s["position"][k])
                arr[i].rotation[k] = float(s.get("rotation", (0, 0, 0))[k])
            w = s.get("width", (0.0, 0.0))
            arr[i].width[0] = float(w[0])
            arr[i].width[1] = float(w[1])
        return arr

    def update_sources(self, sources):
        arr = self.make_sources(sources)
        self.check(self.lib.hrt_update_sources(self.h, len(sources), arr))

    def upload_source_fluxes(self, fluxes):
        f = f32(fluxes).ravel()
        self.check(self.lib.hrt_upload_source_fluxes(self.h, ptr(f), f.size))

    def zero_radiation_buffers(self, nb):
        self.check(self.lib.hrt_zero_radiation_buffers(self.h, nb))

    def zero_scatter_buffers(self):
        self.check(self.lib.hrt_zero_scatter_buffers(self.h))

    def copy_scatter_to_radiation(self):
        self.check(self.lib.hrt_copy_scatter_to_radiation(self.h))

    def upload_radiation_out(self, top, bottom):
        t, b = f32(top).ravel(), f32(bottom).ravel()
        self.check(self.lib.hrt_upload_radiation_out(self.h, ptr(t), ptr(b), t.size))

    def _launch(self, p: dict) -> Launch:
        keep = []

        def a(key, dt):
            v = p.get(key)
            if v is None:
                return None
            arr = np.ascontiguousarray(v, dt).ravel()
            keep.append(arr)
            return ptr(arr)

        L = Launch()
        L.launch_offset = int(p.get("launch_offset", 0))
        L.launch_count = int(p.get("launch_count", self.n))
        L.rays_per_primitive = int(p["rays_per_primitive"])
        L.random_seed = int(p.get("random_seed", 0)) & 0xFFFFFFFF
        L.pass_id = int(p.get("pass_id", 0))
        L.nbands_global = int(p["nbands_global"])
        L.nbands_launch = int(p["nbands_launch"])
        L.band_launch_flag = a("band_launch_flag", np.uint8)
        L.launch_face = int(p.get("launch_face", 1))
        L.diffuse_flux = a("diffuse_flux", np.float32)
        L.diffuse_extinction = a("diffuse_extinction", np.float32)
        L.diffuse_peak_dir = a("diffuse_peak_dir", np.float32)
        L.diffuse_dist_norm = a("diffuse_dist_norm", np.float32)
        L.sky_radiance_params = a("sky_radiance_params", np.float32)
        L.radiation_out_top = a("radiation_out_top", np.float32)
        L.radiation_out_bottom = a("radiation_out_bottom", np.float32)
        self._keep = keep
        return L

    def launch_direct(self, **p):
        L = self._launch(p)
        self.check(self.lib.hrt_launch_direct(self.h, C.byref(L)))

    def launch_diffuse(self, **p):
        L = self._launch(p)
        self.check(self.lib.hrt_launch_diffuse(self.h, C.byref(L)))

    def get_results(self, nb):
        m = self.n * nb
        out = {k: np.zeros(m, np.float32) for k in ("radiation_in", "radiation_out_top", "radiation_out_bottom",
                                                     "scatter_buff_top", "scatter_buff_bottom")}
        self.check(self.lib.hrt_get_results(self.h, ptr(out["radiation_in"]), ptr(out["radiation_out_top"]),
                                            ptr(out["radiation_out_bottom"]), ptr(out["scatter_buff_top"]),
                                            ptr(out["scatter_buff_bottom"])))
        return out

    # -------------------------------------------------------------- whole solve
    def band_solve(self, solve: dict):
        """Build an hrt_band_solve from the same dict the oracle takes; returns (struct, keepalive)."""
        keep = []

        def a(key, dt):
            v = solve.get(key)
            if v is None:
                return None
            arr = np.ascontiguousarray(v, dt).ravel()
            keep.append(arr)
            return ptr(arr)

        s = BandSolve()
        bl = np.ascontiguousarray(solve["band_launch"], np.uint8)
        keep.append(bl)
        s.nbands_global = bl.size
        s.band_launch = ptr(bl)
        srcs = solve.get("sources")
        if srcs is not None:
            arr = self.make_sources(srcs)
            keep.append(arr)
            s.sources = C.cast(arr, C.c_void_p)
            s.nsources = len(srcs)
        else:
            s.sources = None
            s.nsources = int(solve.get("nsources", 0))
        s.source_flux = a("source_flux", np.float32)
        s.rho = a("rho", np.float32)
        s.tau = a("tau", np.float32)
        s.diffuse_flux = a("diffuse_flux", np.float32)
        s.diffuse_extinction = a("diffuse_ext", np.float32)
        s.diffuse_peak_dir = a("diffuse_peak", np.float32)
        s.diffuse_dist_norm = a("diffuse_norm", np.float32)
        s.sky_radiance_params = a("prague", np.float32)
        s.direct_rays = a("direct_rays", np.int32)
        s.diffuse_rays = a("diffuse_rays", np.int32)
        s.scattering_depth = a("depth", np.int32)
        s.emission = a("emission", np.uint8)
        s.emissivity = a("eps", np.float32)
        s.temperature = a("temperature", np.float32)
        s.seed = int(solve.get("seed", 0)) & 0xFFFFFFFF
        s.scatter_tolerance = float(solve.get("scatter_tolerance", 0.0))
        cams = solve.get("cameras") or []
        self.last_cameras = []
        if cams:
            nb = int(np.count_nonzero(np.asarray(solve["band_launch"])))
            arr = (Camera * len(cams))()
            for i, cam in enumerate(cams):
                arr[i] = make_camera(cam)
                W, H = int(cam["resolution"][0]), int(cam["resolution"][1])
                out = {"pixels": np.zeros((H, W, nb), np.float32), "labels": np.zeros((H, W), np.uint32),
                       "depths": np.zeros((H, W), np.float32)}
                arr[i].pixels, arr[i].labels, arr[i].depths = ptr(out["pixels"]), ptr(out["labels"]), ptr(out["depths"])
                self.last_cameras.append(out)
            keep.append(arr)
            s.ncameras = len(cams)
            s.cameras = C.cast(arr, C.c_void_p)
            if solve.get("camera_sky") is not None:
                m = make_sky_model(solve["camera_sky"], keep)
                keep.append(m)
                s.camera_sky = C.cast(C.pointer(m), C.c_void_p)
        return s, keep

    # ---------------------------------------------------------------- cameras
    def update_sky_model(self, nbands, sky=None):
        keep = []
        m = None if sky is None else make_sky_model(sky, keep)
        self.check(self.lib.hrt_update_sky_model(self.h, int(nbands) if sky is not None else 0,
                                                 None if m is None else C.byref(m)))

    def launch_camera(self, cam: dict):
        c = make_camera(cam)
        self.check(self.lib.hrt_launch_camera(self.h, C.byref(c)))

    def launch_pixel_labels(self, cam: dict):
        c = make_camera(cam)
        self.check(self.lib.hrt_launch_pixel_labels(self.h, C.byref(c)))

    def zero_camera_pixel_buffers(self, width, height):
        self.check(self.lib.hrt_zero_camera_pixel_buffers(self.h, int(width), int(height)))

    # --------------------------------------------------------- energy balance
    def energy_balance(self, surf: dict, net_radiation=None, temperature=None, outputs=False):
        """Surface temperatures [n] (and fluxes [n, 5]: sensible, latent, storage, net radiation,
        VPD) of hrt_energy_balance; net_radiation / temperature None use the device-resident ones."""
        keep = []
        s = make_surface(surf, keep)
        n = int(np.asarray(surf["air_temperature"]).size)
        R = None if net_radiation is None else f32(net_radiation).ravel()
        T0 = None if temperature is None else f32(temperature).ravel()
        T = np.zeros(n, np.float32)
        out = np.zeros((n, 5), np.float32) if outputs else None
        self.check(self.lib.hrt_energy_balance(self.h, n, C.byref(s), ptr(R), ptr(T0), ptr(T), ptr(out)))
        return (T, out) if outputs else T

    def run_coupled(self, solve: dict, surf: dict, max_iterations=20, tolerance=1e-3):
        """hrt_run_coupled: (flux [n, Bl], temperature [n], iterations)."""
        self.update_glass(solve.get("is_glass"), solve.get("glass_n"), solve.get("glass_kl"))
        b, keep = self.band_solve(solve)
        s = make_surface(surf, keep)
        bl = int(np.count_nonzero(np.asarray(solve["band_launch"])))
        flux = np.zeros((self.n, bl), np.float32)
        T = np.zeros(self.n, np.float32)
        it = C.c_int32(0)
        self.check(self.lib.hrt_run_coupled(self.h, C.byref(b), C.byref(s), int(max_iterations), float(tolerance),
                                            ptr(flux), ptr(T), C.byref(it)))
        return flux, T, it.value

    def get_camera_results(self, width, height, nbands, pixels=True, labels=True):
        pix = np.zeros((height, width, nbands), np.float32) if pixels else None
        lab = np.zeros((height, width), np.uint32) if labels else None
        dep = np.zeros((height, width), np.float32) if labels else None
        self.check(self.lib.hrt_get_camera_results(self.h, ptr(pix), ptr(lab), ptr(dep), int(width), int(height)))
        return pix, lab, dep

    def run_band(self, solve: dict, out: bool = True, flux_out=None):
        """Device-resident runBand; returns the [n, launched bands] FP32 flux (out=True), written
        into flux_out when given (a C-contiguous float32 array of that shape, e.g. pinned)."""
        self.update_glass(solve.get("is_glass"), solve.get("glass_n"), solve.get("glass_kl"))
        s, keep = self.band_solve(solve)
        bl = int(np.count_nonzero(np.asarray(solve["band_launch"])))
        flux = None
        if out:
            if flux_out is not None:
                if (flux_out.shape != (self.n, bl) or flux_out.dtype != np.float32
                        or not flux_out.flags["C_CONTIGUOUS"]):
                    raise ValueError(f"flux_out must be C-contiguous float32 of shape {(self.n, bl)}")
                flux = flux_out
            else:
                flux = np.zeros((self.n, bl), np.float32)
        self.check(self.lib.hrt_run_band(self.h, C.byref(s), ptr(flux)))
        return flux

    def run_sweep(self, sun_dir, direct_flux, diffuse_flux, rho, tau, direct_rays, diffuse_rays, depth, seed,
                  out=True):
        """Batched solves: returns flux [n, nsun, nbands] (channel c = sun * nbands + band)."""
        sd = f32(sun_dir).reshape(-1, 3)
        nsun = sd.shape[0]
        df = f32(direct_flux).reshape(nsun, -1)
        nb = df.shape[1]
        sk = f32(diffuse_flux).reshape(nsun, nb)
        rh = f32(rho).reshape(self.n, nb)
        ta = f32(tau).reshape(self.n, nb)
        S = Sweep(nsun, ptr(sd), nb, ptr(df), ptr(sk), ptr(rh), ptr(ta), int(direct_rays), int(diffuse_rays),
                  int(depth), int(seed) & 0xFFFFFFFF)
        flux = np.zeros((self.n, nsun, nb), np.float32) if out else None
        self.check(self.lib.hrt_run_sweep(self.h, C.byref(S), ptr(flux)))
        return flux

    def _sweep_struct(self, sun_dir, direct_flux, diffuse_flux, rho, tau, direct_rays, diffuse_rays, depth, seed):
        sd = f32(sun_dir).reshape(-1, 3)
        nsun = sd.shape[0]
        df = f32(direct_flux).reshape(nsun, -1)
        nb = df.shape[1]
        keep = [sd, df, f32(diffuse_flux).reshape(nsun, nb), f32(rho).reshape(self.n, nb), f32(tau).reshape(self.n, nb)]
        S = Sweep(nsun, ptr(keep[0]), nb, ptr(keep[1]), ptr(keep[2]), ptr(keep[3]), ptr(keep[4]), int(direct_rays),
                  int(diffuse_rays), int(depth), int(seed) & 0xFFFFFFFF)
        return S, keep, (self.n, nsun, nb)

    def set_tuning(self, mode: int):
        """1: tune kernel variants per pass shape (default); 0: fixed default; 2: retune."""
        self.check(self.lib.hrt_set_tuning(self.h, int(mode)))

    def set_ray_budget(self, rays_per_thread: int):
        """Rays a thread of the persistent trace takes before its block retires (0: no limit)."""
        self.check(self.lib.hrt_set_ray_budget(self.h, int(rays_per_thread)))

    def set_launch_ray_limit(self, max_rays: int):
        """Rays one trace launch may carry; larger passes run as primitive chunks (tests lower it)."""
        self.check(self.lib.hrt_set_launch_ray_limit(self.h, int(max_rays)))

    def set_visit_budget(self, visits: int):
        """Node visits a ray segment may make before traversal ends it with a device error (0: 2n+64)."""
        self.check(self.lib.hrt_set_visit_budget(self.h, int(visits)))

    def tuning_report(self) -> str:
        k = self.lib.hrt_tuning_report(self.h, None, 0)
        buf = C.create_string_buffer(int(k))
        self.lib.hrt_tuning_report(self.h, buf, k)
        return buf.value.decode()

    def last_stats(self):
        st = np.zeros(4, np.uint64)
        self.check(self.lib.hrt_last_stats(self.h, ptr(st), 4))
        return {"rays": int(st[0]), "kernels": int(st[1]), "iterations": int(st[2]),
                "eb_unconverged": int(st[3])}

    # -------------------------------------------------------------- inspection
    def trace_rays(self, o, d, tmin=1e-4, tmax=1e38, anyhit=False):
        o, d = f32(o).reshape(-1, 3), f32(d).reshape(-1, 3)
        n = o.shape[0]
        hit = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        face = np.zeros(n, np.int32)
        self.check(self.lib.hrt_trace_rays(self.h, n, ptr(o), ptr(d), tmin, tmax, int(anyhit), ptr(hit), ptr(t),
                                           ptr(face)))
        return hit, t, face

    def gen_rays(self, kind, seed, pass_id, rpp, face=1, direction=(0.0, 0.0, 1.0)):
        dimx = max(int(np.sqrt(np.float32(rpp))), 1)
        nr = dimx * (rpp // dimx)
        o = np.zeros((self.n * nr, 3), np.float32)
        d = np.zeros((self.n * nr, 3), np.float32)
        dv = f32(direction)
        self.check(self.lib.hrt_gen_rays(self.h, kind, seed, pass_id, rpp, face, ptr(dv), ptr(o), ptr(d)))
        return o, d

    def bvh(self):
        n = self.n
        codes = np.zeros(n, np.uint64)
        perm = np.zeros(n, np.uint32)
        nodes = np.zeros((max(n - 1, 1), 16), np.uint32)
        self.check(self.lib.hrt_get_bvh(self.h, ptr(codes), ptr(perm), ptr(nodes)))
        return codes, perm, nodes

    def set_measure(self, flags: int):
        self.check(self.lib.hrt_set_measure(self.h, int(flags)))

    def get_measure(self):
        out = np.zeros(10, np.float64)
        self.check(self.lib.hrt_get_measure(self.h, ptr(out), 10))
        return {"direct_launches": int(out[0]), "direct_ms": float(out[1]), "diffuse_launches": int(out[2]),
                "diffuse_ms": float(out[3]), "node_visits": int(out[4]), "prim_tests": int(out[5]),
                "direct_rays": int(out[6]), "diffuse_rays": int(out[7]), "diffuse_node_visits": int(out[8]),
                "diffuse_prim_tests": int(out[9])}

    def device_status(self, reset=True):
        st = C.c_uint32()
        self.check(self.lib.hrt_device_status(self.h, C.byref(st), int(reset)))
        return st.value


def run_sweep_multi(contexts, sweeps, out=True):
    """Sweeps of several scenes in one launch graph (hrt_run_sweep_multi): contexts[k] holds scene
    k, sweeps[k] a dict of Context.run_sweep's arguments (sun_dir, direct_flux, diffuse_flux,
    rho, tau, direct_rays, diffuse_rays, depth, seed).  Returns one flux [n, nsun, nbands] per
    scene; the graph runs on contexts[0]'s stream."""
    lib = load()
    k = len(contexts)
    structs, keep, shapes = (Sweep * k)(), [], []
    for i, (c, sw) in enumerate(zip(contexts, sweeps)):
        S, kp, shape = c._sweep_struct(**sw)
        structs[i] = S
        keep.append(kp)
        shapes.append(shape)
    handles = (VP * k)(*[c.h for c in contexts])
    flux = [np.zeros(sh, np.float32) for sh in shapes] if out else None
    outs = (VP * k)(*[ptr(f) for f in flux]) if out else None
    rc = lib.hrt_run_sweep_multi(handles, structs, k, outs)
    contexts[0].check(rc)
    return flux


class Server:
    """Continuous-batching server over libhrt (hrt_server_*)."""

    def __init__(self, device=0, workers=8, hbm_budget=32 << 30):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.hrt_server_create(C.byref(h), device, workers, int(hbm_budget))
        if rc != HRT_OK:
            raise HrtError(rc, "hrt_server_create failed")
        self.h = h
        self.scenes = {}

    def check(self, rc, what):
        if rc != HRT_OK:
            raise HrtError(rc, what)

    def add_scene(self, scene_id, T, ptype, twosided, rho, tau):
        T = f32(T).reshape(-1, 16)
        ty = np.ascontiguousarray(ptype, np.uint32)
        ts = np.ascontiguousarray(twosided, np.int8)
        rho = f32(rho).reshape(T.shape[0], -1)
        tau = f32(tau).reshape(T.shape[0], -1)
        g = Geometry(T.shape[0], ptr(T), ptr(ty), ptr(ts), 0, None, 0.0, 0.0)
        self.check(self.lib.hrt_server_add_scene(self.h, scene_id, C.byref(g), rho.shape[1], ptr(rho), ptr(tau)),
                   "add_scene")
        self.scenes[scene_id] = (T.shape[0], rho.shape[1])

    def submit(self, request_id, scene_id, arrival_s, band_launch, sun_dir, source_flux, diffuse_flux,
               direct_rays, diffuse_rays, depth, seed, keep=False):
        bl = np.ascontiguousarray(band_launch, np.uint8)
        sf, df = f32(source_flux).ravel(), f32(diffuse_flux).ravel()
        q = ServeRequest(int(request_id), int(scene_id), float(arrival_s), ptr(bl), (C.c_float * 3)(*sun_dir),
                         ptr(sf), ptr(df), int(direct_rays), int(diffuse_rays), int(depth), int(seed) & 0xFFFFFFFF,
                         int(bool(keep)))
        self.check(self.lib.hrt_server_submit(self.h, C.byref(q)), "submit")

    def start(self):
        self.check(self.lib.hrt_server_start(self.h), "start")

    def wait(self):
        self.check(self.lib.hrt_server_wait(self.h), "wait")

    def result(self, request_id, count=0):
        timing = np.zeros(3, np.float64)
        cs = C.c_double()
        rays = C.c_uint64()
        flux = np.zeros(count, np.float32) if count else None
        self.check(self.lib.hrt_server_result(self.h, int(request_id), ptr(flux), count, ptr(timing), C.byref(cs),
                                              C.byref(rays)), "result")
        return {"arrival": timing[0], "admit": timing[1], "done": timing[2], "checksum": cs.value,
                "rays": rays.value, "flux": flux}

    def stats(self):
        out = np.zeros(8, np.float64)
        self.check(self.lib.hrt_server_stats(self.h, ptr(out), 8), "stats")
        return {"builds": int(out[0]), "evictions": int(out[1]), "resident_bytes": out[2], "budget": out[3],
                "batches": int(out[4]), "batched_requests": int(out[5]), "groups": int(out[6]),
                "grouped_batches": int(out[7])}

    def close(self):
        if getattr(self, "h", None):
            self.lib.hrt_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
