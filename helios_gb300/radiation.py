"""Host-side mirror of the reference radiation plugin's user API over libhrt.

``Context`` holds the part of ``helios::Context`` the radiation solve reads
(primitive transforms, types, two-sided flags, primitive and global data);
``RadiationModel`` keeps the method names, argument meaning, defaults and error
behaviour of ``helios::RadiationModel`` (plugins/radiation/include/RadiationModel.h)
for the radiation path: bands, sources, ray counts, scattering depth,
``updateGeometry`` and ``runBand``, whose results land in the primitive data
``radiation_flux_<band>``.

``runBand`` has two execution modes:
  * ``"device"`` (default): one ``hrt_run_band`` call, all passes on the GPU;
  * ``"backend"``: the pass sequence of ``RadiationModel::runBand``
    (src/RadiationModel.cpp:3470-4663) issued call by call through the
    RayTracingBackend-shaped entry points (launchDirectRays, getRadiationResults,
    uploadRadiationOut, ...), exactly as the reference drives a backend.
Both give the same numbers for the same seed.
"""
from __future__ import annotations

import math

import numpy as np

from . import _hrt, scenes

SIGMA = 5.6703744e-8  # RadiationModel.h:2210


class HeliosRuntimeError(RuntimeError):
    """Raised where the reference calls helios_runtime_error (core/include/global.h:102)."""


class Context:
    """Primitive store: transforms, types, two-sided flags, primitive data."""

    def __init__(self):
        self._chunks = []  # (T [k,16] float32, type [k] uint32, area [k] float64)
        self._n = 0
        self._cache = None
        self.primitive_data: dict[str, dict[int, object]] = {}
        self.bulk_data: dict[str, np.ndarray] = {}
        self.global_data: dict[str, object] = {}
        # texture masks: 2-D uint8 arrays (row 0 = top of the image, nonzero = opaque)
        self.masks: list[np.ndarray] = []
        self._mask_index: dict[int, int] = {}
        self.mask_of: dict[int, int] = {}
        self.uv_of: dict[int, np.ndarray] = {}

    # --------------------------------------------------------------- geometry
    def _add_many(self, T, ptype, area):
        T = np.asarray(T, np.float32).reshape(-1, 16)
        k = T.shape[0]
        self._chunks.append((T, np.broadcast_to(np.asarray(ptype, np.uint32), (k,)).copy(),
                             np.broadcast_to(np.asarray(area, np.float64), (k,)).copy()))
        first = self._n
        self._n += k
        self._cache = None
        return first

    def _add(self, T, ptype, area):
        return self._add_many(T, ptype, area)

    def _set_mask(self, uuid, texture_mask, uv):
        if texture_mask is None:
            return
        m = np.ascontiguousarray(texture_mask, np.uint8)
        if m.ndim != 2 or m.size == 0:
            raise HeliosRuntimeError("ERROR (Context): a texture mask is a non-empty 2-D array.")
        k = self._mask_index.get(id(texture_mask))
        if k is None:
            k = len(self.masks)
            self.masks.append(m)
            self._mask_index[id(texture_mask)] = k
        self.mask_of[int(uuid)] = k
        if uv is not None:
            q = np.zeros(8, np.float32)
            uv = np.asarray(uv, np.float32).reshape(-1, 2)
            q[: 2 * len(uv)] = uv.ravel()
            for j in range(len(uv), 4):  # pad to four corners with the last (as the reference does)
                q[2 * j: 2 * j + 2] = uv[-1]
            self.uv_of[int(uuid)] = q

    def addPatch(self, center=(0, 0, 0), size=(1, 1), rotation=(0.0, 0.0), texture_mask=None, uv=None):
        """rotation = (elevation, azimuth) radians, as SphericalCoord(1, elevation, azimuth).
        texture_mask: 2-D array standing in for a texture's transparency channel (row 0 = top,
        nonzero = opaque); uv: texture (u, v) of the corners (-x-y, +x-y, +x+y, -x+y)."""
        if size[0] < 1e-6 or size[1] < 1e-6:
            raise HeliosRuntimeError("ERROR (Context::addPatch): Size of patch must be greater than 1e-6 "
                                     "to avoid numerical precision issues.")
        T = scenes.helios_patch_T(center, size, rotation[0], rotation[1])
        u = self._add(T, scenes.PATCH, size[0] * size[1])
        self._set_mask(u, texture_mask, uv)
        return u

    def addTriangle(self, v0, v1, v2, texture_mask=None, uv=None):
        """texture_mask as for addPatch; uv: texture (u, v) of v0, v1, v2."""
        T = scenes.triangle_T(v0, v1, v2)[0]
        a = 0.5 * np.linalg.norm(np.cross(np.subtract(v1, v0), np.subtract(v2, v0)))
        u = self._add(T, scenes.TRIANGLE, a)
        self._set_mask(u, texture_mask, uv)
        return u

    def mask_arrays(self):
        """Texture masks in the layout of hrt_geometry, or None without masks."""
        if not self.mask_of:
            return None
        n = self._n
        mid = np.full(n, -1, np.int32)
        uvid = np.full(n, -1, np.int32)
        uv = np.zeros((n, 8), np.float32)
        for k, v in self.mask_of.items():
            mid[k] = v
        for k, q in self.uv_of.items():
            uvid[k] = k
            uv[k] = q
        sizes = np.array([[m.shape[1], m.shape[0]] for m in self.masks], np.int32)
        data = np.concatenate([m.ravel() for m in self.masks]).astype(np.uint8)
        return {"mask_id": mid, "uv_id": uvid, "uv": uv, "sizes": sizes, "data": data}

    def addTile(self, center=(0, 0, 0), size=(1, 1), rotation=(0.0, 0.0), div=(1, 1)):
        s = scenes.tile_grid(center, size, div, twosided=1)
        return [self._add(T, scenes.PATCH, a) for T, a in zip(s.T, s.area)]

    def addDisk(self, center, radius, normal=(0, 0, 1)):
        T = scenes.disks(np.asarray(center, np.float64)[None], radius, np.asarray(normal, np.float64)[None])[0]
        return self._add(T, scenes.DISK, math.pi * radius * radius)

    def addVoxel(self, center, size):
        """Voxel primitive; its leaves come from primitive data ``leaf_area_density``
        (m^2/m^3).  Its radiation fluxes are per unit leaf area."""
        T = scenes.voxel_T(np.asarray(center, np.float64)[None], size)[0]
        return self._add(T, scenes.VOXEL, 2 * (size[0] * size[1] + size[1] * size[2] + size[0] * size[2]))

    def addPrimitives(self, T, ptype, area=None, twosided=None):
        """Bulk add (synthetic scenes): returns the new UUIDs."""
        T = np.asarray(T, np.float32).reshape(-1, 16)
        first = self._add_many(T, ptype, 1.0 if area is None else area)
        uuids = np.arange(first, first + T.shape[0])
        if twosided is not None:
            self.setPrimitiveData(uuids, "twosided_flag", np.broadcast_to(np.asarray(twosided, np.float64), uuids.shape))
        return uuids

    # ------------------------------------------------------------ file input
    def _add_loaded(self, f):
        """Add the primitives of a loaded file (helios_gb300._hrt.load_scene_file)."""
        T, ty = f["T"].astype(np.float64), f["type"]
        c0, c1, c2 = T[:, [0, 4, 8]], T[:, [1, 5, 9]], T[:, [2, 6, 10]]
        a, b, c = (np.linalg.norm(x, axis=1) for x in (c0, c1, c2))
        cr = np.linalg.norm(np.cross(c0, c1), axis=1)
        area = np.select([ty == scenes.TRIANGLE, ty == 2, ty == 4], [0.5 * cr, math.pi * a * b, 2.0 * (a * b + b * c + c * a)],
                         cr)
        uu = self.addPrimitives(f["T"], ty, area, f["twosided"])
        for lab, v in f["data"].items():
            m = ~np.isnan(v)
            if m.any():
                self.setPrimitiveData(uu[m], lab, v[m])
        return uu

    def loadPLY(self, filename, origin=(0.0, 0.0, 0.0), height=0.0, rotation=(0.0, 0.0), default_color=(0.0, 0.0, 1.0),
                upaxis="YUP"):
        """Context::loadPLY (core/src/Context_fileIO.cpp:3617-3908): triangles of a PLY file
        (rotation = (elevation, azimuth)); returns their UUIDs."""
        if not str(filename).lower().endswith(".ply"):
            raise HeliosRuntimeError(f"ERROR (Context::loadPLY): File {filename} is not PLY format.")
        return self._load_file(filename, origin, height, rotation, default_color, upaxis, "loadPLY")

    def loadOBJ(self, filename, origin=(0.0, 0.0, 0.0), height=0.0, rotation=(0.0, 0.0), default_color=(0.0, 0.0, 1.0),
                upaxis="ZUP"):
        """Context::loadOBJ (core/src/Context_fileIO.cpp:3983-4340): triangles of an OBJ file."""
        if not str(filename).lower().endswith(".obj"):
            raise HeliosRuntimeError(f"ERROR (Context::loadOBJ): File {filename} is not OBJ format.")
        return self._load_file(filename, origin, height, rotation, default_color, upaxis, "loadOBJ")

    def loadXML(self, filename):
        """Context::loadXML (core/src/Context_fileIO.cpp:1260-2230): patches, triangles, voxels
        and disks with their transforms and scalar primitive data."""
        if not str(filename).lower().endswith(".xml"):
            raise HeliosRuntimeError(f"failed.\n File {filename} is not XML format.")
        return self._load_file(filename, (0, 0, 0), 0.0, (0, 0), (0, 0, 1), "ZUP", "loadXML")

    def _load_file(self, filename, origin, height, rotation, color, upaxis, fn):
        from . import _hrt
        try:
            f = _hrt.load_scene_file(filename, origin, height, rotation, upaxis, color)
        except (ValueError, _hrt.HrtError) as e:
            raise HeliosRuntimeError(f"ERROR (Context::{fn}): {e}") from None
        return self._add_loaded(f)

    def addScene(self, sc: "scenes.Scene"):
        uuids = self.addPrimitives(sc.T, sc.ptype, sc.area, sc.twosided)
        if sc.lad is not None:
            self.setPrimitiveData(uuids, "leaf_area_density", np.asarray(sc.lad, np.float64))
        return uuids

    def getPrimitiveCount(self):
        return self._n

    def getAllUUIDs(self):
        return list(range(self._n))

    def getPrimitiveArea(self, uuid):
        return float(self.arrays()[2][uuid])

    def arrays(self):
        if self._cache is None:
            if self._chunks:
                T = np.concatenate([c[0] for c in self._chunks])
                ty = np.concatenate([c[1] for c in self._chunks])
                area = np.concatenate([c[2] for c in self._chunks])
                self._chunks = [(T, ty, area)]
            else:
                T, ty, area = np.zeros((0, 16), np.float32), np.zeros(0, np.uint32), np.zeros(0)
            self._cache = (T, ty, area)
        return self._cache

    def getDomainBoundingBox(self):
        """x, y, z bounds over all primitive vertices (Context::getDomainBoundingBox)."""
        T, ty, _ = self.arrays()
        if T.shape[0] == 0:
            return (0.0, 0.0), (0.0, 0.0), (0.0, 0.0)
        lo = np.full(3, np.inf)
        hi = np.full(3, -np.inf)
        ax, ay, c = T[:, [0, 4, 8]].astype(np.float64), T[:, [1, 5, 9]].astype(np.float64), T[:, [3, 7, 11]].astype(np.float64)
        corners = {scenes.PATCH: ((-0.5, -0.5), (0.5, -0.5), (0.5, 0.5), (-0.5, 0.5)),
                   scenes.TILE: ((-0.5, -0.5), (0.5, -0.5), (0.5, 0.5), (-0.5, 0.5)),
                   scenes.TRIANGLE: ((0, 0), (0, 1), (1, 1))}
        for t, cs in corners.items():
            m = ty == t
            for cx, cy in cs:
                p = ax[m] * cx + ay[m] * cy + c[m]
                if p.size:
                    lo = np.minimum(lo, p.min(0))
                    hi = np.maximum(hi, p.max(0))
        m = ty == scenes.DISK
        if m.any():
            r = np.linalg.norm(ax[m], axis=1)[:, None]
            lo = np.minimum(lo, (c[m] - r).min(0))
            hi = np.maximum(hi, (c[m] + r).max(0))
        m = ty == scenes.VOXEL
        if m.any():
            h = 0.5 * np.abs(np.stack([T[m, 0], T[m, 5], T[m, 10]], 1))
            lo = np.minimum(lo, (c[m] - h).min(0))
            hi = np.maximum(hi, (c[m] + h).max(0))
        return (lo[0], hi[0]), (lo[1], hi[1]), (lo[2], hi[2])

    # --------------------------------------------------------------- data
    def setPrimitiveData(self, uuid, label, value):
        if np.ndim(uuid) > 0 and np.asarray(value).dtype.kind in "US":  # strings: one entry per primitive
            uuids = np.asarray(uuid).ravel()
            vals = np.broadcast_to(np.asarray(value), uuids.shape)
            d = self.primitive_data.setdefault(label, {})
            for u, v in zip(uuids.tolist(), vals.tolist()):
                d[int(u)] = str(v)
            return
        if np.ndim(uuid) > 0:
            uuids = np.asarray(uuid).ravel()
            vals = np.broadcast_to(np.asarray(value), uuids.shape)
            arr = self._bulk(label, vals.dtype)
            arr[uuids] = vals
            d = self.primitive_data.get(label)
            if d:  # values set one by one earlier are replaced
                for u in uuids.tolist():
                    d.pop(u, None)
            return
        d = self.primitive_data.setdefault(label, {})
        d[int(uuid)] = value
        if label in self.bulk_data:
            self._bulk(label, np.asarray(value).dtype)[int(uuid)] = value

    def _bulk(self, label, dtype):
        n = self._n
        arr = self.bulk_data.get(label)
        if arr is None or arr.shape[0] < n:
            new = np.full(n, np.nan, np.float64)
            if arr is not None:
                new[: arr.shape[0]] = arr
            for k, v in self.primitive_data.get(label, {}).items():
                new[k] = v
            self.bulk_data[label] = arr = new
        return arr

    def doesPrimitiveDataExist(self, uuid, label):
        if label in self.bulk_data and uuid < self.bulk_data[label].shape[0]:
            return not np.isnan(self.bulk_data[label][uuid])
        return uuid in self.primitive_data.get(label, {})

    def getPrimitiveData(self, uuid, label):
        if label in self.bulk_data and uuid < self.bulk_data[label].shape[0]:
            v = self.bulk_data[label][uuid]
            if not np.isnan(v):
                return float(v)
        d = self.primitive_data.get(label, {})
        if uuid not in d:
            raise HeliosRuntimeError(f"ERROR (Context::getPrimitiveData): Primitive data {label} does not exist "
                                     f"for primitive {uuid}.")
        return d[uuid]

    def primitive_array(self, label, default):
        """Dense float64 view of a primitive-data label with a default for missing entries."""
        n = self._n
        out = np.full(n, float(default))
        if label in self.bulk_data:
            a = self.bulk_data[label][:n]
            m = ~np.isnan(a)
            out[: a.shape[0]][m] = a[m]
        for k, v in self.primitive_data.get(label, {}).items():
            if k < n:
                out[k] = float(v)
        return out

    def setGlobalData(self, label, value):
        self.global_data[label] = value

    def getGlobalData(self, label):
        return self.global_data[label]

    def doesGlobalDataExist(self, label):
        return label in self.global_data


def _interp_clamped(x, xs, ys):
    """Piecewise-linear value at x, clamped to the end values (RadiationModel.cpp:3312-3366)."""
    if x <= xs[0]:
        return ys[0]
    if x >= xs[-1]:
        return ys[-1]
    i = max(int(np.searchsorted(np.asarray(xs, np.float32), np.float32(x), side="left")), 1)
    t = np.float32((np.float32(x) - np.float32(xs[i - 1])) / (np.float32(xs[i]) - np.float32(xs[i - 1])))
    return float(np.float32(ys[i - 1]) + t * (np.float32(ys[i]) - np.float32(ys[i - 1])))


def _spectrum_over_band(spec, w1, w2, source=None):
    """Band value of an object spectrum [(wavelength, value)] over [w1, w2]
    (RadiationModel::integrateSpectrum, RadiationModel.cpp:1463-1538), in FP32: the trapezoids
    run over the object's own wavelengths from the segment holding w1 to the one holding w2.
    With a source spectrum: sum value x source / sum source, the source interpolated at the
    object's wavelengths (clamped at its ends).  Without one the source is taken as flat: the
    integral divided by (w2 - w1), which the caller does (RadiationModel.cpp:2450)."""
    f = np.float32
    n = len(spec)
    if n < 2 or not w1 < w2:
        raise HeliosRuntimeError("ERROR (RadiationModel::integrateSpectrum): Radiation spectrum must have at least 2 "
                                 "wavelengths and the lower wavelength bound must be less than the upper one.")
    xs = [f(x) for x, _ in spec]
    ys = [f(y) for _, y in spec]
    istart, iend = (0 if source is not None else 1), n - 1
    for i in range(n - 1):
        if xs[i] <= w1 < xs[i + 1]:
            istart = i
        if xs[i] <= w2 < xs[i + 1]:
            iend = i + 1
            break
    if source is None:
        E = f(0.0)
        for i in range(istart, iend):
            E = f(E + f(f(f(ys[i] + ys[i + 1]) * f(xs[i + 1] - xs[i])) * f(0.5)))
        return float(E)
    sx = [w for w, _ in source]
    sy = [v for _, v in source]
    E = Etot = f(0.0)
    for i in range(istart, iend):
        s0, s1 = f(_interp_clamped(xs[i], sx, sy)), f(_interp_clamped(xs[i + 1], sx, sy))
        dx = f(xs[i + 1] - xs[i])
        E = f(E + f(f(f(0.5) * f(f(ys[i] * s0) + f(ys[i + 1] * s1))) * dx))
        Etot = f(Etot + f(f(f(0.5) * f(s1 + s0)) * dx))
    return float(f(E / Etot))


def _weighted_average(wl, values, weights, response):
    """Radiance-weighted mean of a unitless spectral parameter over a response curve:
    sum p L R dl / sum L R dl by trapezoids over the response's segments
    (RadiationModel::weightedAverageOverResponse, RadiationModel.cpp:3290-3380)."""
    if not wl or not response:
        return 0.0
    num = den = 0.0
    for (l1, r1), (l2, r2) in zip(response[:-1], response[1:]):
        if l2 < wl[0] or l1 > wl[-1]:
            continue
        p1, p2 = _interp_clamped(l1, wl, values), _interp_clamped(l2, wl, values)
        w1, w2 = _interp_clamped(l1, wl, weights), _interp_clamped(l2, wl, weights)
        dl = l2 - l1
        num += 0.5 * (p1 * w1 * r1 + p2 * w2 * r2) * dl
        den += 0.5 * (w1 * r1 + w2 * r2) * dl
    return float(np.float32(num / den)) if den > 1e-10 else 0.0


def _angular_normalization(circ, width, horiz, N=50):
    """1 / integral of the Prague pattern x cos(theta) over the hemisphere with the sun at the
    zenith, midpoint rule on N x N cells in FP32 (RadiationModel::computeAngularNormalization,
    RadiationModel.cpp:3382-3414)."""
    f = np.float32
    i = np.arange(N, dtype=np.float32)
    theta = f(0.5) * f(math.pi) * (i + f(0.5)) / f(N)
    cos_t = np.maximum(f(0.0), np.cos(theta).astype(np.float32))  # dir.z with the sun at the zenith
    gamma = np.arccos(np.clip(cos_t, -1, 1)).astype(np.float32) * f(180.0) / f(math.pi)
    pattern = (f(1.0) + f(circ) * np.exp(-gamma / f(width)).astype(np.float32)) * \
        (f(1.0) + (f(horiz) - f(1.0)) * (f(1.0) - cos_t))
    w = pattern * np.cos(theta).astype(np.float32) * np.sin(theta).astype(np.float32) * \
        (f(math.pi) / (f(2.0) * f(N))) * (f(2.0) * f(math.pi) / f(N))
    integral = f(0.0)
    for _ in range(N):  # the azimuth loop adds the same column N times, in FP32
        for v in w:
            integral = f(integral + v)
    return float(f(1.0) / max(integral, f(1e-10)))


class _Band:
    def __init__(self):
        self.directRayCount = 100       # RadiationModel.cpp:40
        self.diffuseRayCount = 1000     # RadiationModel.cpp:41
        self.diffuseFlux = -1.0         # RadiationModel.cpp:43
        self.scatteringDepth = 0        # RadiationModel.cpp:46
        self.emissionFlag = True        # RadiationModel.h:549
        self.diffuseExtinction = 0.0
        self.diffusePeakDir = (0.0, 0.0, 1.0)
        self.diffuseDistNorm = 1.0
        self.wavebandBounds = (0.0, 0.0)  # RadiationModel.h RadiationBand::wavebandBounds
        self.diffuse_spectrum = []        # [(wavelength, value)]
        self.diffusePragueParams = (0.0, 0.0, 0.0, 0.0)  # circumsolar strength, width (deg), horizon, norm


class RadiationModel:
    def __init__(self, context: Context, device: int = 0, mode: str = "device"):
        self.context = context
        self.device = device
        self._ctx = None
        self.mode = mode
        self.bands: dict[str, _Band] = {}
        self.sources: list[dict] = []
        self.periodic = (0.0, 0.0)
        self.seed = 0
        self.auto_seed = True
        self.message_flag = True
        self._geom_n = -1
        self.rho_default, self.tau_default, self.eps_default = 0.0, 0.0, 1.0
        self.temperature_default = 300.0
        self.scatter_tolerance = 0.0
        self.last_stats = {}
        self.cameras: dict[str, dict] = {}
        self.camera_sky_radiance: dict[str, float] = {}

    @property
    def ctx(self) -> "_hrt.Context":
        """The device context, created on first use (initialize(), RayTracingBackend.h:54)."""
        if self._ctx is None:
            self._ctx = _hrt.Context(self.device)
        return self._ctx

    # --------------------------------------------------------------- config
    def disableMessages(self):
        self.message_flag = False

    def setSeed(self, seed: int):
        """Fix the Philox key of the next runBand calls (the reference seeds from the clock)."""
        self.seed = int(seed) & 0xFFFFFFFF
        self.auto_seed = False

    def addRadiationBand(self, label, wavelength_min=None, wavelength_max=None):
        if label in self.bands:
            raise HeliosRuntimeError(f"ERROR (RadiationModel::addRadiationBand): Radiation band {label} has already "
                                     "been added.")
        band = _Band()
        if wavelength_min is not None and wavelength_max is not None:
            band.wavebandBounds = (float(wavelength_min), float(wavelength_max))
        band.diffuse_spectrum = list(getattr(self, "_global_diffuse_spectrum", []))
        self.bands[label] = band
        for s in self.sources:
            s["fluxes"].setdefault(label, -1.0)

    def doesBandExist(self, label):
        return label in self.bands

    def _band(self, label, fn):
        if label not in self.bands:
            raise HeliosRuntimeError(f"ERROR (RadiationModel::{fn}): Cannot {fn} for band '{label}' because it "
                                     "is not a valid band.")
        return self.bands[label]

    # -------------------------------------------------------------- cameras
    def addRadiationCamera(self, label, band_labels, position, lookat, properties=None, antialiasing_samples=1):
        """A radiation camera (RadiationCamera.cpp:30-88).  properties: dict with the
        CameraProperties fields this solve uses -- camera_resolution (512, 512),
        focal_plane_distance 1, lens_diameter 0.05, HFOV 20 degrees, camera_zoom 1.  Pixel data
        is radiance (the reference's "manual" exposure); exposure and white balance are not
        applied."""
        p = {"camera_resolution": (512, 512), "focal_plane_distance": 1.0, "lens_diameter": 0.05, "HFOV": 20.0,
             "camera_zoom": 1.0}
        p.update(properties or {})
        W, H = int(p["camera_resolution"][0]), int(p["camera_resolution"][1])
        if int(antialiasing_samples) == 0:
            raise HeliosRuntimeError("ERROR (RadiationModel::addRadiationCamera): The model requires at least 1 "
                                     "antialiasing sample to run.")
        if W <= 0 or H <= 0:
            raise HeliosRuntimeError("ERROR (RadiationModel::addRadiationCamera): Camera resolution must be at "
                                     "least 1x1.")
        if p["HFOV"] < 0 or p["HFOV"] > 180.0:
            raise HeliosRuntimeError("ERROR (RadiationModel::addRadiationCamera): Camera horizontal field of view "
                                     "must be between 0 and 180 degrees.")
        self.cameras[label] = {"bands": list(band_labels), "position": tuple(map(float, position)),
                               "lookat": tuple(map(float, lookat)), "props": p, "aa": int(antialiasing_samples),
                               "pixels": {}, "labels": None, "depths": None}

    def setCameraSkyRadiance(self, band, radiance):
        """Sky radiance cameras see on a miss that meets no source, for one band.  The reference
        computes it with its atmospheric sky model (RadiationModel.cpp:2928-3050), which runs only
        when atmospheric global data are set; this sets its output directly (default 0)."""
        self.camera_sky_radiance[band] = float(radiance)

    @staticmethod
    def _view_direction(position, lookat):
        """(zenith, azimuth) of lookat - position as cart2sphere gives them (global.cpp:818-831)."""
        d = np.asarray(lookat, np.float32) - np.asarray(position, np.float32)
        r = np.float32(math.sqrt(float(d[0]) ** 2 + float(d[1]) ** 2 + float(d[2]) ** 2))
        x, y = float(d[0]), float(d[1])
        if abs(x) < 1e-7 and abs(y) < 1e-7:
            y = 1e-7
        elev = math.asin(max(-1.0, min(1.0, float(d[2]) / float(r))))
        az = math.atan2(x, y)
        if az < 0:
            az += 2.0 * math.pi
        return 0.5 * math.pi - elev, az

    def _camera_dicts(self, band_labels, seed):
        """Cameras whose bands meet this dispatch (RadiationModel.cpp:4431-4448), in label order."""
        out, labels = [], []
        for cid, (label, cam) in enumerate(sorted(self.cameras.items())):
            if not any(b in band_labels for b in cam["bands"]):
                continue
            p = cam["props"]
            W, H = int(p["camera_resolution"][0]), int(p["camera_resolution"][1])
            hfov = float(p["HFOV"]) / float(p["camera_zoom"])
            zen, az = self._view_direction(cam["position"], cam["lookat"])
            out.append({"position": cam["position"], "direction": (zen, az),
                        "focal_length": float(p["focal_plane_distance"]), "lens_diameter": float(p["lens_diameter"]),
                        "fov_aspect": float(np.float32(W) / np.float32(H)),
                        "viewplane_length": float(0.5 / math.tan(0.5 * hfov * math.pi / 180.0)),
                        "resolution": (W, H), "antialiasing": cam["aa"], "seed": seed, "camera_id": cid})
            labels.append(label)
        return out, labels

    def _camera_sky_dict(self, band_labels):
        """The camera sky of a dispatch (the updateSkyModel inputs, RadiationModel.cpp:4368-4428):
        Prague parameters (none in this mirror), the sky radiance, the first collimated or
        sun-sphere source as the solar disk (collimated: flux / 6.74e-5 sr; sun sphere: flux / pi;
        cos 0.999989), and the sky flux of every band with its emission flag."""
        sky = {"sky_radiance": np.array([self.camera_sky_radiance.get(b, 0.0) for b in band_labels], np.float32),
               "prague": np.zeros((len(band_labels), 4), np.float32), "sun": (0.0, 0.0, 1.0), "disk_cos": 0.0,
               "disk_radiance": np.zeros(len(band_labels), np.float32),
               "diffuse_flux": np.array([self.getDiffuseFlux(b) for b in band_labels], np.float32),
               "emission": np.array([1 if self.bands[b].emissionFlag else 0 for b in band_labels], np.uint32)}
        for k, src in enumerate(self.sources):
            if src["type"] in (0, 2):
                v = np.asarray(src["position"], np.float32)
                sky["sun"] = tuple(float(x) for x in v / np.float32(math.sqrt(float(np.dot(v, v)))))
                fl = np.array([self.getSourceFlux(k, b) for b in band_labels], np.float32)
                sky["disk_radiance"] = (fl / np.float32(math.pi) if src["type"] == 2 else fl / np.float32(6.74e-5))
                sky["disk_cos"] = 0.999989
                break
        return sky

    def getCameraPixelData(self, label, band):
        if label not in self.cameras:
            raise HeliosRuntimeError(f"ERROR (RadiationModel::getCameraPixelData): Camera '{label}' does not exist.")
        if band not in self.cameras[label]["pixels"]:
            raise HeliosRuntimeError(f"ERROR (RadiationModel::getCameraPixelData): Band '{band}' has no pixel data "
                                     f"for camera '{label}'.")
        return self.cameras[label]["pixels"][band]

    def getCameraPixelLabels(self, label):
        return self.cameras[label]["labels"]

    def getCameraPixelDepths(self, label):
        return self.cameras[label]["depths"]

    def disableEmission(self, label):
        self._band(label, "disableEmission").emissionFlag = False

    def enableEmission(self, label):
        self._band(label, "enableEmission").emissionFlag = True

    def setDirectRayCount(self, label, n):
        self._band(label, "setDirectRayCount").directRayCount = int(n)

    def setDiffuseRayCount(self, label, n):
        self._band(label, "setDiffuseRayCount").diffuseRayCount = int(n)

    def setScatteringDepth(self, label, depth):
        if depth < 0:
            raise HeliosRuntimeError("ERROR (RadiationModel::setScatteringDepth): scattering depth must be >= 0.")
        self._band(label, "setScatteringDepth").scatteringDepth = int(depth)

    def setDiffuseRadiationFlux(self, label, flux):
        self._band(label, "setDiffuseRadiationFlux").diffuseFlux = float(flux)

    def setDiffuseRadiationExtinctionCoeff(self, label, K, peak_direction):
        """Power-law sky fd = psi^-K normalised over the hemisphere (RadiationModel.cpp:185-217)."""
        b = self._band(label, "setDiffuseRadiationExtinctionCoeff")
        d = np.asarray(peak_direction, np.float64)
        d = d / np.linalg.norm(d)
        N = 100
        th = 0.5 * math.pi / N * (0.5 + np.arange(N))
        ph = 2.0 * math.pi / N * (0.5 + np.arange(N))
        TH, PH = np.meshgrid(th, ph, indexing="ij")
        el = 0.5 * math.pi - TH  # sphere2cart(elevation, azimuth) convention
        v = np.stack([np.cos(el) * np.sin(PH), np.cos(el) * np.cos(PH), np.sin(el)], -1)
        psi = np.arccos(np.clip(v @ d, -1.0, 1.0))
        fd = np.where(psi < math.pi / 180.0, (math.pi / 180.0) ** (-K), psi ** (-K))
        norm = float((fd * np.cos(TH) * np.sin(TH) * math.pi / (N * N)).sum())
        b.diffuseExtinction = float(K)
        b.diffusePeakDir = tuple(d)
        b.diffuseDistNorm = 1.0 / norm

    def setDiffuseSpectrum(self, spectrum_label):
        """Diffuse spectrum of every band (and of bands added later) from global data of
        (wavelength, value) pairs (RadiationModel.cpp:1287-1310).  A manual diffuse flux still
        wins (getDiffuseFlux); the spectrum weights the Prague sky parameters."""
        if not self.context.doesGlobalDataExist(spectrum_label):
            raise HeliosRuntimeError(f"ERROR (RadiationModel::setDiffuseSpectrum): Global data '{spectrum_label}' "
                                     "does not exist.")
        spec = [(float(w), float(v)) for w, v in self.context.getGlobalData(spectrum_label)]
        self._global_diffuse_spectrum = spec
        for b in self.bands.values():
            b.diffuse_spectrum = list(spec)

    def setSourceSpectrum(self, source, spectrum_label):
        """Spectrum of one or more sources from global data of (wavelength, value) pairs
        (RadiationModel::setSourceSpectrum); it weights the band averages of primitive spectra."""
        if not self.context.doesGlobalDataExist(spectrum_label):
            raise HeliosRuntimeError(f"ERROR (RadiationModel::setSourceSpectrum): Global data '{spectrum_label}' "
                                     "does not exist.")
        spec = [(float(w), float(v)) for w, v in self.context.getGlobalData(spectrum_label)]
        for sid in (np.atleast_1d(source).tolist()):
            if sid >= len(self.sources):
                raise HeliosRuntimeError("ERROR (RadiationModel::setSourceSpectrum): Source ID out of bounds.")
            self.sources[int(sid)]["spectrum"] = spec

    def _spectral_property(self, kind, bands, S):
        """[S][n][Bg] values of primitives whose `<kind>_spectrum` names global spectral data, NaN
        elsewhere (RadiationModel.cpp:2400-2470, 2625-2700): per band with waveband bounds and
        per source, the spectrum averaged over the band, weighted by the source's spectrum if it
        has one, else flat; NaN for bands without bounds (the constant value applies)."""
        labels = self.context.primitive_data.get(kind + "_spectrum", {})
        n = self.context.getPrimitiveCount()
        out = np.full((S, n, len(bands)), np.nan)
        if not labels:
            return out
        cache = {}
        ptype = self.context.arrays()[1]
        for uuid, lab in labels.items():
            if not isinstance(lab, str) or not self.context.doesGlobalDataExist(lab):
                continue
            if ptype[uuid] == scenes.VOXEL:  # voxels take no spectra (RadiationModel.cpp:2626)
                continue
            for bi, b in enumerate(bands):
                w1, w2 = self.bands[b].wavebandBounds
                if w1 == 0 or w2 == 0:
                    continue
                for si in range(S):
                    src = self.sources[si].get("spectrum")
                    key = (lab, b, si if src else -1)
                    if key not in cache:
                        spec = [(float(w), float(v)) for w, v in self.context.getGlobalData(lab)]
                        cache[key] = (_spectrum_over_band(spec, w1, w2, src) if src else
                                      _spectrum_over_band(spec, w1, w2) / (w2 - w1))
                    out[si, uuid, bi] = cache[key]
        return out

    def _update_prague(self, band_labels):
        """Prague sky parameters of the general diffuse radiation from the Context's global data
        (RadiationModel::updatePragueParametersForGeneralDiffuse, RadiationModel.cpp:3145-3223):
        with prague_sky_valid == 1, every band without a power-law sky gets the circumsolar
        strength, circumsolar width and horizon brightness of prague_sky_spectral_params (6 values
        per wavelength) averaged over its diffuse spectrum (or waveband) weighted by the zenith
        radiance, the normalisation recomputed from them, and the sun direction as peak."""
        g = self.context
        if not g.doesGlobalDataExist("prague_sky_valid") or int(g.getGlobalData("prague_sky_valid")) != 1:
            return
        sp = np.asarray(g.getGlobalData("prague_sky_spectral_params"), np.float32).reshape(-1)
        nw = sp.size // 6
        sp = sp[:6 * nw].reshape(nw, 6)
        wl, Lz = sp[:, 0].tolist(), sp[:, 1].tolist()
        sun = tuple(float(x) for x in g.getGlobalData("prague_sky_sun_direction"))
        for label in band_labels:
            band = self.bands[label]
            if band.diffuseExtinction > 0.0:
                continue
            spec = band.diffuse_spectrum
            if not spec:
                lo, hi = band.wavebandBounds
                if lo > 0 and hi > lo:
                    spec = [(lo, 1.0), (hi, 1.0)]
            if not spec:
                continue
            circ = _weighted_average(wl, sp[:, 2].tolist(), Lz, spec)
            width = _weighted_average(wl, sp[:, 3].tolist(), Lz, spec)
            horiz = _weighted_average(wl, sp[:, 4].tolist(), Lz, spec)
            band.diffusePragueParams = (circ, width, horiz, _angular_normalization(circ, width, horiz))
            band.diffusePeakDir = sun

    def _add_source(self, src):
        if len(self.sources) >= 256:
            raise HeliosRuntimeError("ERROR (RadiationModel): A maximum of 256 radiation sources are allowed.")
        src["fluxes"] = {b: -1.0 for b in self.bands}
        self.sources.append(src)
        return len(self.sources) - 1

    def addCollimatedRadiationSource(self, direction=(0.0, 0.0, 1.0)):
        d = np.asarray(direction, np.float64)
        if np.linalg.norm(d) == 0:
            raise HeliosRuntimeError("ERROR (RadiationModel::addCollimatedRadiationSource): Invalid collimated "
                                     "source direction. Direction vector should not have length of zero.")
        return self._add_source({"type": 0, "position": tuple(d), "width": (0.0, 0.0), "rotation": (0, 0, 0)})

    def addSunSphereRadiationSource(self, direction=(0.0, 0.0, 1.0)):
        d = np.asarray(direction, np.float64)
        d = 150e9 * d / np.linalg.norm(d)
        return self._add_source({"type": 2, "position": tuple(d), "width": (2 * 695.5e6, 0.0), "rotation": (0, 0, 0)})

    def addSphereRadiationSource(self, position, radius):
        return self._add_source({"type": 1, "position": tuple(position), "width": (2 * radius, 0.0),
                                 "rotation": (0, 0, 0)})

    def addRectangleRadiationSource(self, position, size, rotation):
        return self._add_source({"type": 3, "position": tuple(position), "width": tuple(size),
                                 "rotation": tuple(rotation)})

    def addDiskRadiationSource(self, position, radius, rotation):
        return self._add_source({"type": 4, "position": tuple(position), "width": (radius, 0.0),
                                 "rotation": tuple(rotation)})

    def setSourceFlux(self, source, label, flux):
        self._band(label, "setSourceFlux")
        if source >= len(self.sources):
            raise HeliosRuntimeError("ERROR (RadiationModel::setSourceFlux): Source ID out of bounds.")
        self.sources[source]["fluxes"][label] = float(flux)

    def getSourceFlux(self, source, label):
        f = self.sources[source]["fluxes"].get(label, -1.0)
        return 0.0 if f < 0 else f  # RadiationModel.cpp:1226-1230

    def getDiffuseFlux(self, label):
        f = self.bands[label].diffuseFlux
        return f if f >= 0 else 0.0  # RadiationModel.cpp:1312-1330

    def enforcePeriodicBoundary(self, boundary):
        px, py = self.periodic
        if boundary == "x":
            px = 1.0
        elif boundary == "y":
            py = 1.0
        elif boundary == "xy":
            px = py = 1.0
        else:
            print(f"WARNING (RadiationModel::enforcePeriodicBoundary()): unknown boundary of '{boundary}'. "
                  "Possible choices are x, y, or xy.")
        self.periodic = (px, py)
        self._geom_n = -1

    # --------------------------------------------------------------- geometry
    def _bbox_faces(self):
        px, py = self.periodic
        if px != 1 and py != 1:
            return None
        (x0, x1), (y0, y1), (z0, z1) = self.context.getDomainBoundingBox()
        x0, x1, y0, y1, z0, z1 = (np.float32(v) for v in (x0 - 1e-5, x1 + 1e-5, y0 - 1e-5, y1 + 1e-5, z0 - 1e-5,
                                                            z1 + 1e-5))
        faces = []
        if px == 1:  # RadiationModel.cpp:6046-6063
            faces.append([(x0, y0, z0), (x0, y1, z0), (x0, y1, z1), (x0, y0, z1)])
            faces.append([(x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1)])
        if py == 1:
            faces.append([(x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1)])
            faces.append([(x0, y1, z0), (x1, y1, z0), (x1, y1, z1), (x0, y1, z1)])
        return np.asarray(faces, np.float32)

    def setScatteringResidualTolerance(self, tol: float):
        """Stop a band's scattering iterations once the FP64 residual (power scattered by
        the last iteration over the band's total) is at most ``tol``; 0 (the default) runs
        every iteration up to the scattering depth, as the reference does.  No counterpart
        in the reference."""
        if not tol >= 0.0:
            raise HeliosRuntimeError("ERROR (RadiationModel::setScatteringResidualTolerance): tolerance must be >= 0.")
        self.scatter_tolerance = float(tol)

    def voxel_lad(self):
        """Leaf area density of every primitive (read for voxels, primitive data
        ``leaf_area_density``), or None when the context holds no voxels."""
        _, ty, _ = self.context.arrays()
        if not (ty == scenes.VOXEL).any():
            return None
        return self.context.primitive_array("leaf_area_density", 0.0).astype(np.float32)

    def geometry_arrays(self):
        T, ty, area = self.context.arrays()
        ts = self.context.primitive_array("twosided_flag", 1).astype(np.int8)
        ts[ty == scenes.VOXEL] = 1  # a voxel launches both directions of each sample
        keep = (area > 0) | (ty == scenes.TILE)  # zero-area primitives are skipped (RadiationModel.cpp:5813-5824)
        if not keep.all():
            raise HeliosRuntimeError("zero-area primitives are not supported by this mirror")
        return T, ty, ts

    def updateGeometry(self):
        T, ty, ts = self.geometry_arrays()
        self._ts = ts
        self.ctx.update_geometry(T, ty, ts, self._bbox_faces(), self.periodic, self.voxel_lad(),
                                 self.context.mask_arrays())
        self.ctx.build_accel()
        self._geom_n = T.shape[0]

    # --------------------------------------------------------------- solve
    def _materials(self, band_labels, S):
        """rho/tau [S][N][Bg] and eps [N][Bl] following updateRadiativeProperties (RadiationModel.cpp:2850-2880)."""
        n = self.context.getPrimitiveCount()
        all_bands = sorted(self.bands)
        Bg = len(all_bands)
        rho = np.zeros((S, n, Bg))
        tau = np.zeros((S, n, Bg))
        eps_l = np.ones((n, len(band_labels)))
        self._glass = None
        # spectral reflectivity / transmissivity: used where no constant (other than the default)
        # is set for the band (RadiationModel.cpp:2640-2660), clamped to [0, 1]
        rho_spec = self._spectral_property("reflectivity", all_bands, S)
        tau_spec = self._spectral_property("transmissivity", all_bands, S)
        for bi, b in enumerate(all_bands):
            band = self.bands[b]
            r0 = self.context.primitive_array("reflectivity_" + b, self.rho_default)
            t0 = self.context.primitive_array("transmissivity_" + b, self.tau_default)
            e = self.context.primitive_array("emissivity_" + b, self.eps_default)
            r_s = np.clip(np.where((r0 == self.rho_default) & ~np.isnan(rho_spec[:, :, bi]), rho_spec[:, :, bi], r0), 0, 1)
            t_s = np.clip(np.where((t0 == self.tau_default) & ~np.isnan(tau_spec[:, :, bi]), tau_spec[:, :, bi], t0), 0, 1)
            r, t = r_s[0], t_s[0]
            # translucent cover: glass_n_<band> >= 1 activates the sheet model, glass_KL_<band>
            # (default 0, negative clamped) its absorption (RadiationModel.cpp:2759-2807); the
            # constant rho/tau of a glass entry are kept as set and not checked (:2844-2846)
            gn = self.context.primitive_array("glass_n_" + b, np.nan)
            g = gn >= 1.0
            if g.any():
                if self._glass is None:
                    self._glass = (np.zeros((n, Bg), np.int8), np.zeros((n, Bg), np.float32),
                                   np.zeros((n, Bg), np.float32))
                gkl = np.maximum(self.context.primitive_array("glass_KL_" + b, 0.0), 0.0)
                self._glass[0][:, bi] = g
                self._glass[1][:, bi] = np.where(g, gn, 0.0)
                self._glass[2][:, bi] = np.where(g, gkl, 0.0)
            if band.emissionFlag:
                m1 = ~g & (e != 1.0) & (r == 0) & (t == 0)
                r = np.where(m1, 1.0 - e, r)
                bad = ~g & ~m1 & (np.abs(e + t + r - 1.0) > 1e-6) & (e > 0)
                if bad.any():
                    raise HeliosRuntimeError(f"ERROR (RadiationModel): emissivity, transmissivity, and reflectivity "
                                             f"must sum to 1 to ensure energy conservation. Band {b}. It is also "
                                             "possible that you forgot to disable emission for this band.")
                m3 = ~g & ~m1 & (band.scatteringDepth == 0) & (e != 1.0)
                e = np.where(m3, 1.0, e)
                r = np.where(m3, 0.0, r)
                t = np.where(m3, 0.0, t)
            elif (~g & (t + r > 1.0 + 1e-6)).any():
                raise HeliosRuntimeError("ERROR (RadiationModel): transmissivity and reflectivity cannot sum to "
                                         "greater than 1 ensure energy conservation.")
            # the emissivity rules above act on source 0's values; sources with their own spectra
            # keep their spectral values where the rules left a primitive unchanged
            same_r, same_t = r == r_s[0], t == t_s[0]
            rho[:, :, bi] = np.where(same_r[None, :], r_s, r[None, :])
            tau[:, :, bi] = np.where(same_t[None, :], t_s, t[None, :])
            if b in band_labels:
                eps_l[:, band_labels.index(b)] = e
        return rho.astype(np.float32), tau.astype(np.float32), eps_l.astype(np.float32)

    def solve_description(self, labels, seed=None):
        """The band set of one runBand call as plain arrays (shared with the oracle)."""
        if isinstance(labels, str):
            labels = [labels]
        for b in labels:
            if b not in self.bands:
                raise HeliosRuntimeError(f"ERROR (RadiationModel::runBand): Cannot run band {b} because it is not a "
                                         "valid band. Use addRadiationBand() function to add the band.")
        all_bands = sorted(self.bands)  # std::map order (RadiationModel.cpp:3520-3527)
        band_labels = [b for b in all_bands if b in labels]
        self._update_prague(band_labels)  # RadiationModel.cpp:3726-3729
        if not self.sources:
            self.addCollimatedRadiationSource()
        S = len(self.sources)
        rho, tau, eps = self._materials(band_labels, S)
        n = self.context.getPrimitiveCount()
        temp = self.context.primitive_array("temperature", self.temperature_default)
        temp = np.where(temp < 0, self.temperature_default, temp).astype(np.float32)
        sflux = np.array([[self.getSourceFlux(s, b) for b in band_labels] for s in range(S)], np.float32)
        B = [self.bands[b] for b in band_labels]
        desc = {
            "band_labels": band_labels,
            "band_launch": np.array([1 if b in band_labels else 0 for b in all_bands], np.uint8),
            "sources": [dict(s) for s in self.sources],
            "source_flux": sflux,
            "rho": rho, "tau": tau,
            "diffuse_flux": np.array([self.getDiffuseFlux(b) for b in band_labels], np.float32),
            "diffuse_ext": np.array([x.diffuseExtinction for x in B], np.float32),
            "diffuse_norm": np.array([x.diffuseDistNorm for x in B], np.float32),
            "diffuse_peak": np.array([x.diffusePeakDir for x in B], np.float32),
            "prague": np.array([x.diffusePragueParams for x in B], np.float32).reshape(len(B), 4),
            "direct_rays": np.array([x.directRayCount for x in B], np.int32),
            "diffuse_rays": np.array([x.diffuseRayCount for x in B], np.int32),
            "depth": np.array([x.scatteringDepth for x in B], np.int32),
            "emission": np.array([1 if x.emissionFlag else 0 for x in B], np.uint8),
            "eps": eps, "temperature": temp,
            "seed": self.seed if seed is None else seed,
            "scatter_tolerance": self.scatter_tolerance,
            "n": n,
        }
        if self.cameras:
            cams, labels = self._camera_dicts(band_labels, desc["seed"])
            if cams:
                desc["cameras"] = cams
                desc["camera_labels"] = labels
                desc["camera_sky"] = self._camera_sky_dict(band_labels)
        if self._glass is not None:
            desc["is_glass"] = np.ascontiguousarray(np.broadcast_to(self._glass[0], (S, n, len(all_bands))))
            desc["glass_n"] = np.ascontiguousarray(np.broadcast_to(self._glass[1], (S, n, len(all_bands))))
            desc["glass_kl"] = np.ascontiguousarray(np.broadcast_to(self._glass[2], (S, n, len(all_bands))))
        return desc

    def runBand(self, labels):
        if isinstance(labels, str):
            labels = [labels]
        for b in self.bands:
            self.context.setGlobalData("emission_enabled_" + b, 1 if self.bands[b].emissionFlag else 0)
        if self.context.getPrimitiveCount() == 0:
            print("WARNING (RadiationModel::runBand): No geometry was added to the context. There is nothing to "
                  "simulate...exiting.")
            return
        if self._geom_n != self.context.getPrimitiveCount():
            self.updateGeometry()
        desc = self.solve_description(labels)
        if self.mode == "backend":
            flux = run_band_through_backend(self.ctx, desc, self._ts)
        else:
            flux = self.ctx.run_band(desc)
            self.last_stats = self.ctx.last_stats()
        n = desc["n"]
        uu = np.arange(n)
        for i, b in enumerate(desc["band_labels"]):
            self.context.setPrimitiveData(uu, "radiation_flux_" + b, flux[:, i].astype(np.float64))
        self._store_cameras(desc, self.ctx.last_cameras if desc.get("cameras") else [])
        if self.auto_seed:
            self.seed = (self.seed + 0x9E3779B9) & 0xFFFFFFFF
        return flux

    def _store_cameras(self, desc, outs):
        """Pixel data, labels and depths of the rendered cameras as the reference stores them
        (global data camera_<label>_<band>, _pixel_UUID, _pixel_depth; RadiationModel.cpp:4527-4605).
        Labels are primitive UUID + 1 (0 = sky)."""
        for label, out in zip(desc.get("camera_labels", []), outs):
            cam = self.cameras[label]
            H, W = out["labels"].shape
            for i, b in enumerate(desc["band_labels"]):
                px = out["pixels"][:, :, i].reshape(-1).astype(np.float32)
                cam["pixels"][b] = px
                self.context.setGlobalData(f"camera_{label}_{b}", px)
            cam["labels"] = out["labels"].reshape(-1).copy()
            cam["depths"] = out["depths"].reshape(-1).copy()
            self.context.setGlobalData(f"camera_{label}_pixel_UUID", cam["labels"])
            self.context.setGlobalData(f"camera_{label}_pixel_depth", cam["depths"])

    def getTotalAbsorbedFlux(self):
        """Per-primitive sum over bands of radiation_flux_<band> times area (RadiationModel.cpp:4686-4708)."""
        n = self.context.getPrimitiveCount()
        _, _, area = self.context.arrays()
        tot = np.zeros(n)
        for b in self.bands:
            lab = "radiation_flux_" + b
            if lab in self.context.bulk_data:
                tot += np.nan_to_num(self.context.bulk_data[lab][:n]) * area
        return tot


def run_band_through_backend(ctx: "_hrt.Context", d: dict, twosided: np.ndarray) -> np.ndarray:
    """RadiationModel::runBand's pass sequence through the backend entry points
    (src/RadiationModel.cpp:3779-4356 and 4628-4663)."""
    n = d["n"]
    flags = d["band_launch"]
    Bg = flags.size
    Bl = int(flags.sum())
    S = len(d["sources"])
    ctx.update_materials(d["rho"], d["tau"], S, Bg)
    ctx.update_glass(d.get("is_glass"), d.get("glass_n"), d.get("glass_kl"))
    ctx.update_sources(d["sources"])
    scattering = bool((d["depth"] > 0).any())
    diffuse = bool((d["diffuse_flux"] > 0).any())
    emission = bool(d["emission"].any())
    dirN, difN, depth = int(d["direct_rays"].max()), int(d["diffuse_rays"].max()), int(d["depth"].max())
    seed = d["seed"]
    ctx.zero_radiation_buffers(Bl)
    cams = d.get("cameras") or []
    # camera view of the primitives, accumulated on the host as RadiationModel::runBand does
    ctop = np.zeros((n, Bl)) if cams else None
    cbot = np.zeros((n, Bl)) if cams else None

    def cam_add(res):
        if cams:
            ctop[...] += res["scatter_buff_top"].reshape(n, Bl)
            cbot[...] += res["scatter_buff_bottom"].reshape(n, Bl)
    rundirect = bool((d["source_flux"] > 0).any())
    ctx.upload_source_fluxes(d["source_flux"])
    common = dict(launch_offset=0, launch_count=n, random_seed=seed, nbands_global=Bg, nbands_launch=Bl)
    if S > 0 and rundirect:
        ctx.launch_direct(rays_per_primitive=dirN, pass_id=0, band_launch_flag=flags, **common)
    ftop = np.zeros((n, Bl), np.float32)
    fbot = np.zeros((n, Bl), np.float32)
    if scattering and rundirect:
        res = ctx.get_results(Bl)
        cam_add(res)
        ftop = res["scatter_buff_top"].reshape(n, Bl).copy()
        fbot = res["scatter_buff_bottom"].reshape(n, Bl).copy()
        one = twosided == 0
        tot = ftop[one] + fbot[one]
        ftop[one] = tot
        fbot[one] = tot
        ctx.upload_radiation_out(ftop, fbot)
        ctx.zero_scatter_buffers()
    sky = dict(diffuse_extinction=d["diffuse_ext"], diffuse_peak_dir=d["diffuse_peak"],
               diffuse_dist_norm=d["diffuse_norm"], sky_radiance_params=d["prague"])
    rpp = int(math.ceil(math.sqrt(difN))) ** 2
    if emission or diffuse:
        if emission:
            for b in range(Bl):
                if not d["emission"][b]:
                    continue
                e = d["eps"][:, b].copy()
                if d["depth"][b] == 0:
                    e[e != 1.0] = 1.0
                T = d["temperature"].astype(np.float64)
                out = ((SIGMA_F32 * e).astype(np.float64) * (T * T * T * T)).astype(np.float32)
                ftop[:, b] += out
                fbot[twosided != 0, b] += out[twosided != 0]
                if cams:
                    ctop[:, b] += out
                    cbot[twosided != 0, b] += out[twosided != 0]
        for face in (1, 0):
            ctx.launch_diffuse(rays_per_primitive=rpp, pass_id=1, band_launch_flag=flags, launch_face=face,
                               diffuse_flux=d["diffuse_flux"], radiation_out_top=ftop, radiation_out_bottom=fbot,
                               **sky, **common)
        if cams:
            cam_add(ctx.get_results(Bl))
    if scattering and (emission or diffuse) and not rundirect:
        ctx.copy_scatter_to_radiation()
        ctx.zero_scatter_buffers()
    if scattering and (emission or diffuse or rundirect):
        zero = np.zeros(Bl, np.float32)
        sflags = flags.copy()
        for it in range(depth):
            b = -1
            for bg in range(Bg):
                if not sflags[bg]:
                    continue
                b += 1
                if it + 1 > d["depth"][b]:
                    sflags[bg] = 0
            if it > 0 or (emission and rundirect):
                ctx.copy_scatter_to_radiation()
            ctx.zero_scatter_buffers()
            res = ctx.get_results(Bl)
            for face in (1, 0):
                ctx.launch_diffuse(rays_per_primitive=rpp, pass_id=2 + it, band_launch_flag=sflags, launch_face=face,
                                   diffuse_flux=zero, radiation_out_top=res["radiation_out_top"],
                                   radiation_out_bottom=res["radiation_out_bottom"], **sky, **common)
            if cams:
                cam_add(ctx.get_results(Bl))
    res = ctx.get_results(Bl)
    flux = (res["radiation_in"] + res["scatter_buff_top"] + res["scatter_buff_bottom"]).reshape(n, Bl)
    # cameras (RadiationModel.cpp:4358-4616): launchCameraRays / launchPixelLabelRays per camera
    ctx.last_cameras = []
    if cams:
        render = scattering and (emission or diffuse or rundirect)
        if render:
            ctx.upload_radiation_out(ctop.astype(np.float32), cbot.astype(np.float32))
            ctx.update_sky_model(Bl, d.get("camera_sky"))
        for cam in cams:
            W, H = cam["resolution"]
            out = {"pixels": np.zeros((H, W, Bl), np.float32), "labels": np.zeros((H, W), np.uint32),
                   "depths": np.zeros((H, W), np.float32)}
            if render:
                ctx.launch_camera(cam)
                out["pixels"] = ctx.get_camera_results(W, H, Bl, labels=False)[0]
                ctx.zero_camera_pixel_buffers(W, H)
                ctx.launch_pixel_labels(cam)
                _, out["labels"], out["depths"] = ctx.get_camera_results(W, H, Bl, pixels=False)
            ctx.last_cameras.append(out)
    return flux


SIGMA_F32 = np.float32(SIGMA)
