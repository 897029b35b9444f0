"""Seeded synthetic scenes for the radiation solve.

Every generator returns plain numpy arrays in the layout the reference's
``RadiationModel::buildGeometryData`` hands to a ray-tracing backend
(``plugins/radiation/src/RadiationModel.cpp:5808-6148``): one row-major 4x4
FP32 transform per primitive (the Context's ``getPrimitiveTransformationMatrix``
convention), a primitive type code and a two-sided flag.

Canonical shapes (``plugins/radiation/src/optix8/OptiX8DeviceCode.cu:369-489``):
  * patch / tile: the square [-0.5, 0.5]^2 in the local xy plane;
  * triangle: vertices (0,0,0), (0,1,0), (1,1,0);
  * disk: the unit disk in the local xy plane;
  * voxel: the cube [-0.5, 0.5]^3.

The random streams are numpy PCG64 generators seeded by the caller (seed 0 for
the benchmark workloads), never Helios's ``Context::randu``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

PATCH, TRIANGLE, DISK, TILE, VOXEL = 0, 1, 2, 3, 4


@dataclass
class Scene:
    T: np.ndarray                 # [n, 16] float32
    ptype: np.ndarray             # [n] uint32
    twosided: np.ndarray          # [n] int8
    area: np.ndarray              # [n] float64 (one face)
    groups: dict = field(default_factory=dict)   # name -> index array
    bbox_verts: np.ndarray | None = None         # periodic walls [nb, 4, 3]
    periodic: tuple = (0.0, 0.0)
    lad: np.ndarray | None = None                # [n] leaf area density of voxels (0 elsewhere)

    @property
    def n(self) -> int:
        return int(self.T.shape[0])


def _rot(axis: str, a: float) -> np.ndarray:
    c, s = math.cos(a), math.sin(a)
    if axis == "x":
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    if axis == "y":
        return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])


def helios_patch_T(center, size, elevation=0.0, azimuth=0.0) -> np.ndarray:
    """Transform of ``Context::addPatch(center, size, SphericalCoord(1, elevation, azimuth))``:
    scale, rotate(-elevation, x), rotate(-azimuth, z), translate
    (``core/src/Context_primitive.cpp:36-56``)."""
    M = np.diag([float(size[0]), float(size[1]), 1.0])
    if elevation != 0:
        M = _rot("x", -elevation) @ M
    if azimuth != 0:
        M = _rot("z", -azimuth) @ M
    T = np.eye(4)
    T[:3, :3] = M
    T[:3, 3] = center
    return T.reshape(16).astype(np.float32)


def frame_T(center, sx, sy, normal, spin) -> np.ndarray:
    """Vectorised patch transforms: local x/y axes scaled by (sx, sy), local z = unit normal."""
    normal = np.asarray(normal, np.float64)
    normal = normal / np.linalg.norm(normal, axis=-1, keepdims=True)
    helper = np.where(np.abs(normal[..., 2:3]) < 0.9, np.array([0.0, 0.0, 1.0]), np.array([1.0, 0.0, 0.0]))
    ex = np.cross(helper, normal)
    ex /= np.linalg.norm(ex, axis=-1, keepdims=True)
    ey = np.cross(normal, ex)
    c, s = np.cos(spin)[..., None], np.sin(spin)[..., None]
    ex, ey = c * ex + s * ey, -s * ex + c * ey
    n = normal.shape[0]
    T = np.zeros((n, 4, 4))
    T[:, :3, 0] = ex * np.asarray(sx).reshape(-1, 1)
    T[:, :3, 1] = ey * np.asarray(sy).reshape(-1, 1)
    T[:, :3, 2] = normal
    T[:, :3, 3] = center
    T[:, 3, 3] = 1.0
    return T.reshape(n, 16).astype(np.float32)


def triangle_T(v0, v1, v2) -> np.ndarray:
    """Transforms mapping the canonical triangle (0,0,0),(0,1,0),(1,1,0) onto (v0, v1, v2)
    (the mapping ``Triangle::makeTransformationMatrix`` solves for,
    ``core/src/Context_primitive.cpp:1327``)."""
    v0, v1, v2 = (np.asarray(v, np.float64).reshape(-1, 3) for v in (v0, v1, v2))
    n = v0.shape[0]
    nrm = np.cross(v1 - v0, v2 - v0)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=-1, keepdims=True), 1e-30)
    T = np.zeros((n, 4, 4))
    T[:, :3, 0] = v2 - v1
    T[:, :3, 1] = v1 - v0
    T[:, :3, 2] = nrm
    T[:, :3, 3] = v0
    T[:, 3, 3] = 1.0
    return T.reshape(n, 16).astype(np.float32)


def uniform_sphere(rng, n) -> np.ndarray:
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * math.pi, n)
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=-1)


def _concat(parts):
    T = np.concatenate([p[0] for p in parts]).astype(np.float32)
    ty = np.concatenate([np.full(p[0].shape[0], p[1], np.uint32) for p in parts])
    ts = np.concatenate([np.full(p[0].shape[0], p[2], np.int8) for p in parts])
    area = np.concatenate([p[3] for p in parts])
    return T, ty, ts, area


def homogeneous_canopy(n_leaves=20000, leaf=0.1, domain=10.0, zlo=1.0, zhi=3.0, seed=0, ground_div=1,
                       ground_margin=0.0) -> Scene:
    """One-sided ground (one patch, or a ground_div x ground_div tile) + two-sided square
    leaves with a spherical leaf-angle distribution, centres uniform in [0,domain]^2 x [zlo,zhi].
    ground_margin extends the ground past the leaf domain on every side (so that leaves
    overhanging the edge still have ground below them)."""
    rng = np.random.default_rng(seed)
    gs = domain + 2.0 * ground_margin
    if ground_div == 1:
        ground = helios_patch_T((0.5 * domain, 0.5 * domain, 0.0), (gs, gs))[None, :]
    else:
        ground = tile_grid((0.5 * domain, 0.5 * domain, 0.0), (gs, gs), (ground_div, ground_div)).T
    ng = ground.shape[0]
    c = np.stack([rng.uniform(0, domain, n_leaves), rng.uniform(0, domain, n_leaves),
                  rng.uniform(zlo, zhi, n_leaves)], axis=-1)
    nrm = uniform_sphere(rng, n_leaves)
    spin = rng.uniform(0, 2 * math.pi, n_leaves)
    leaves = frame_T(c, np.full(n_leaves, leaf), np.full(n_leaves, leaf), nrm, spin)
    T, ty, ts, area = _concat([(ground, PATCH, 0, np.full(ng, gs * gs / ng)),
                               (leaves, PATCH, 1, np.full(n_leaves, leaf * leaf))])
    return Scene(T, ty, ts, area, {"ground": np.arange(ng), "leaves": np.arange(ng, ng + n_leaves)})


def orchard(nx=20, ny=10, spacing=5.0, leaves_per_tree=5000, side=0.03, radii=(1.5, 1.5, 2.0),
            centre_z=3.0, seed=0, ground=False) -> Scene:
    """Equilateral triangular leaves uniform in ellipsoidal crowns on a regular grid."""
    rng = np.random.default_rng(seed)
    ntree = nx * ny
    n = ntree * leaves_per_tree
    # uniform points in the unit ball
    d = uniform_sphere(rng, n) * (rng.uniform(0, 1, n) ** (1.0 / 3.0))[:, None]
    tx = (np.arange(ntree) % nx) * spacing
    ty_ = (np.arange(ntree) // nx) * spacing
    tid = np.repeat(np.arange(ntree), leaves_per_tree)
    c = np.stack([tx[tid] + radii[0] * d[:, 0], ty_[tid] + radii[1] * d[:, 1], centre_z + radii[2] * d[:, 2]], -1)
    nrm = uniform_sphere(rng, n)
    spin = rng.uniform(0, 2 * math.pi, n)
    # equilateral triangle of side `side` centred at c in the plane normal to nrm
    helper = np.where(np.abs(nrm[:, 2:3]) < 0.9, np.array([0.0, 0.0, 1.0]), np.array([1.0, 0.0, 0.0]))
    ex = np.cross(helper, nrm)
    ex /= np.linalg.norm(ex, axis=-1, keepdims=True)
    ey = np.cross(nrm, ex)
    R = side / math.sqrt(3.0)
    verts = []
    for k in range(3):
        a = spin + 2.0 * math.pi * k / 3.0
        verts.append(c + R * (np.cos(a)[:, None] * ex + np.sin(a)[:, None] * ey))
    T = triangle_T(verts[0], verts[1], verts[2])
    area = np.full(n, math.sqrt(3.0) / 4.0 * side * side)
    parts = [(T, TRIANGLE, 1, area)]
    groups = {"leaves": np.arange(n)}
    if ground:
        gx, gy = nx * spacing, ny * spacing
        g = helios_patch_T((0.5 * gx - 0.5 * spacing, 0.5 * gy - 0.5 * spacing, 0.0), (gx, gy))[None, :]
        parts.append((g, PATCH, 0, np.array([gx * gy])))
        groups["ground"] = np.array([n])
    Tm, tym, tsm, aream = _concat(parts)
    return Scene(Tm, tym, tsm, aream, groups)


def parallel_rectangles(a=1.0, b=2.0, c=0.5) -> Scene:
    """Two one-sided a x b rectangles facing each other at distance c
    (reference selfTest "Black/Gray Parallel Rectangles")."""
    T0 = helios_patch_T((0, 0, 0), (a, b))
    T1 = helios_patch_T((0, 0, c), (a, b), elevation=math.pi, azimuth=0.0)
    T = np.stack([T0, T1])
    return Scene(T, np.zeros(2, np.uint32), np.zeros(2, np.int8), np.full(2, a * b))


def common_edge_squares() -> Scene:
    """Horizontal unit square and a vertical one sharing an edge
    (reference selfTest "90 Degree Common-Edge Squares")."""
    T0 = helios_patch_T((0, 0, 0), (1, 1))
    T1 = helios_patch_T((0.5, 0, 0.5), (1, 1), elevation=0.5 * math.pi, azimuth=-0.5 * math.pi)
    T = np.stack([T0, T1])
    return Scene(T, np.zeros(2, np.uint32), np.zeros(2, np.int8), np.ones(2))


def tile_grid(center=(0.0, 0.0, 0.0), size=(10.0, 10.0), div=(40, 40), twosided=0) -> Scene:
    """A horizontal tile split into div[0] x div[1] patches (``Context::addTile``)."""
    nx, ny = div
    dx, dy = size[0] / nx, size[1] / ny
    xs = center[0] - 0.5 * size[0] + (np.arange(nx) + 0.5) * dx
    ys = center[1] - 0.5 * size[1] + (np.arange(ny) + 0.5) * dy
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    T = np.stack([helios_patch_T((x, y, center[2]), (dx, dy)) for x, y in zip(X.ravel(), Y.ravel())])
    n = T.shape[0]
    return Scene(T, np.zeros(n, np.uint32), np.full(n, twosided, np.int8), np.full(n, dx * dy))


def disks(centers, radius, normals) -> np.ndarray:
    """Transforms of disks (unit disk scaled by radius) with the given normals."""
    n = centers.shape[0]
    spin = np.zeros(n)
    return frame_T(centers, np.full(n, radius), np.full(n, radius), normals, spin)


def voxel_T(centers, size) -> np.ndarray:
    n = centers.shape[0]
    T = np.zeros((n, 4, 4))
    T[:, 0, 0] = size[0]
    T[:, 1, 1] = size[1]
    T[:, 2, 2] = size[2]
    T[:, :3, 3] = centers
    T[:, 3, 3] = 1.0
    return T.reshape(n, 16).astype(np.float32)


def voxel_grid(lo, hi, div, lad) -> Scene:
    """div[0] x div[1] x div[2] axis-aligned voxels filling the box [lo, hi]; lad is a
    scalar or an array of div[0]*div[1]*div[2] leaf area densities (x fastest)."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    nx, ny, nz = div
    size = (hi - lo) / np.array([nx, ny, nz], np.float64)
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    idx = np.stack([ix.ravel(order="F"), iy.ravel(order="F"), iz.ravel(order="F")], -1)
    centers = lo + (idx + 0.5) * size
    n = centers.shape[0]
    T = voxel_T(centers, size)
    lad = np.broadcast_to(np.asarray(lad, np.float64), (n,)).astype(np.float32)
    vol = float(np.prod(size))
    return Scene(T, np.full(n, VOXEL, np.uint32), np.ones(n, np.int8), lad.astype(np.float64) * vol,
                 {"voxels": np.arange(n)}, lad=lad)


def disk_leaves(centers, normals, radius) -> np.ndarray:
    """Disk leaves of one radius centred at `centers` with the given normals."""
    return disks(np.asarray(centers, np.float64), radius, normals)


def concat_scenes(*parts: Scene) -> Scene:
    """Primitives of several scenes in order; groups are renamed <i>:<name> and shifted."""
    T = np.concatenate([p.T for p in parts]).astype(np.float32)
    ty = np.concatenate([p.ptype for p in parts]).astype(np.uint32)
    ts = np.concatenate([p.twosided for p in parts]).astype(np.int8)
    area = np.concatenate([p.area for p in parts])
    lad = np.concatenate([p.lad if p.lad is not None else np.zeros(p.n, np.float32) for p in parts])
    groups, off = {}, 0
    for i, p in enumerate(parts):
        for k, v in p.groups.items():
            groups[f"{i}:{k}"] = np.asarray(v) + off
        off += p.n
    return Scene(T, ty, ts, area, groups, lad=lad if (ty == VOXEL).any() else None)


def deep_scatter(n_tri=3_000_000, n_patch=500_000, n_disk=500_000, vox_div=64, domain=24.0, height=4.0,
                 tri_side=0.03, patch_side=0.04, disk_radius=0.02, lad_max=2.0, seed=0) -> Scene:
    """Deep-scattering stress scene: a one-sided ground patch under two-sided leaves --
    n_tri equilateral triangles, n_patch square patches and n_disk disks (spherical leaf
    angles, centres uniform in [0, domain]^2 x [0.05, height]) -- and a vox_div^3 voxel
    grid over the same box with leaf area density uniform in [0, lad_max]."""
    rng = np.random.default_rng(seed)

    def centres(k):
        return np.stack([rng.uniform(0, domain, k), rng.uniform(0, domain, k), rng.uniform(0.05, height, k)], -1)

    c = centres(n_tri)
    nrm = uniform_sphere(rng, n_tri)
    spin = rng.uniform(0, 2 * math.pi, n_tri)
    helper = np.where(np.abs(nrm[:, 2:3]) < 0.9, np.array([0.0, 0.0, 1.0]), np.array([1.0, 0.0, 0.0]))
    ex = np.cross(helper, nrm)
    ex /= np.linalg.norm(ex, axis=-1, keepdims=True)
    ey = np.cross(nrm, ex)
    R = tri_side / math.sqrt(3.0)
    vs = [c + R * (np.cos(spin + 2 * math.pi * k / 3)[:, None] * ex + np.sin(spin + 2 * math.pi * k / 3)[:, None] * ey)
          for k in range(3)]
    tris = Scene(triangle_T(vs[0], vs[1], vs[2]), np.full(n_tri, TRIANGLE, np.uint32), np.ones(n_tri, np.int8),
                 np.full(n_tri, math.sqrt(3.0) / 4.0 * tri_side * tri_side), {"triangles": np.arange(n_tri)})
    c = centres(n_patch)
    Tp = frame_T(c, np.full(n_patch, patch_side), np.full(n_patch, patch_side), uniform_sphere(rng, n_patch),
                 rng.uniform(0, 2 * math.pi, n_patch))
    patches = Scene(Tp, np.full(n_patch, PATCH, np.uint32), np.ones(n_patch, np.int8),
                    np.full(n_patch, patch_side * patch_side), {"patches": np.arange(n_patch)})
    c = centres(n_disk)
    Td = disk_leaves(c, uniform_sphere(rng, n_disk), disk_radius)
    dsk = Scene(Td, np.full(n_disk, DISK, np.uint32), np.ones(n_disk, np.int8),
                np.full(n_disk, math.pi * disk_radius * disk_radius), {"disks": np.arange(n_disk)})
    nv = vox_div ** 3
    vox = voxel_grid((0.0, 0.0, 0.0), (domain, domain, height), (vox_div, vox_div, vox_div),
                     rng.uniform(0.0, lad_max, nv))
    ground = Scene(helios_patch_T((0.5 * domain, 0.5 * domain, 0.0), (domain, domain))[None, :],
                   np.array([PATCH], np.uint32), np.zeros(1, np.int8), np.array([domain * domain]),
                   {"ground": np.array([0])})
    sc = concat_scenes(ground, tris, patches, dsk, vox)
    sc.groups = {"ground": np.array([0]), "triangles": 1 + np.arange(n_tri),
                 "patches": 1 + n_tri + np.arange(n_patch), "disks": 1 + n_tri + n_patch + np.arange(n_disk),
                 "voxels": 1 + n_tri + n_patch + n_disk + np.arange(nv)}
    return sc


def sun_direction(zenith_deg: float, azimuth_deg: float) -> np.ndarray:
    """Unit vector toward the sun, Helios ``sphere2cart`` convention (azimuth from +y toward +x,
    ``core/src/global.cpp:833``)."""
    el = math.radians(90.0 - zenith_deg)
    az = math.radians(azimuth_deg)
    return np.array([math.cos(el) * math.sin(az), math.cos(el) * math.cos(az), math.sin(el)], np.float32)


def day_sweep(latitude_deg=38.5, day_of_year=180, n=96, bands=("PAR", "NIR")):
    """Sun positions every 24h/n of local solar time (Cooper's declination, hour angle) and a
    simple clear-sky split per band: direct normal flux S*k^(1/sin(elev)-1) and isotropic
    sky flux f*S*sin(elev), both zero with the sun below the horizon.
    Returns (sun_dir [n,3] toward the sun, direct [n,B], diffuse [n,B], elevation [n] rad)."""
    params = {"PAR": (500.0, 0.75, 0.15), "NIR": (450.0, 0.80, 0.10)}
    lat = math.radians(latitude_deg)
    dec = math.radians(23.45) * math.sin(2.0 * math.pi * (284 + day_of_year) / 365.0)
    dirs, direct, diffuse, elev = [], [], [], []
    for k in range(n):
        hour = 24.0 * k / n
        w = math.radians(15.0 * (hour - 12.0))
        se = math.sin(lat) * math.sin(dec) + math.cos(lat) * math.cos(dec) * math.cos(w)
        el = math.asin(max(-1.0, min(1.0, se)))
        # azimuth from north toward east
        az = math.atan2(-math.sin(w) * math.cos(dec),
                        math.cos(lat) * math.sin(dec) - math.sin(lat) * math.cos(dec) * math.cos(w))
        dirs.append([math.cos(el) * math.sin(az), math.cos(el) * math.cos(az), math.sin(el)])
        row_d, row_s = [], []
        for b in bands:
            S, kk, f = params[b]
            if se > 1e-3:
                row_d.append(S * kk ** (1.0 / se - 1.0))
                row_s.append(f * S * se)
            else:
                row_d.append(0.0)
                row_s.append(0.0)
        direct.append(row_d)
        diffuse.append(row_s)
        elev.append(el)
    return (np.asarray(dirs, np.float32), np.asarray(direct, np.float32), np.asarray(diffuse, np.float32),
            np.asarray(elev))


def mixed_canopy(n, lai, seed=0, height=3.0, leaf_area=0.0025):
    """Homogeneous canopy of n leaves, half square patches and half equilateral triangles
    (patch:triangle 1:1) of equal area, spherical leaf angles, over a one-sided ground
    patch; the domain side follows from the leaf area index: sqrt(n * leaf_area / LAI)."""
    rng = np.random.default_rng(seed)
    n_patch = n // 2
    n_tri = n - n_patch
    dom = math.sqrt(max(n, 1) * leaf_area / lai)
    side_p = math.sqrt(leaf_area)
    side_t = math.sqrt(4.0 * leaf_area / math.sqrt(3.0))
    c = np.stack([rng.uniform(0, dom, n), rng.uniform(0, dom, n), rng.uniform(0.05, height, n)], -1)
    nrm = uniform_sphere(rng, n)
    spin = rng.uniform(0, 2 * math.pi, n)
    Tp = frame_T(c[:n_patch], np.full(n_patch, side_p), np.full(n_patch, side_p), nrm[:n_patch], spin[:n_patch])
    ct, nt, st = c[n_patch:], nrm[n_patch:], spin[n_patch:]
    helper = np.where(np.abs(nt[:, 2:3]) < 0.9, np.array([0.0, 0.0, 1.0]), np.array([1.0, 0.0, 0.0]))
    ex = np.cross(helper, nt)
    ex /= np.linalg.norm(ex, axis=-1, keepdims=True)
    ey = np.cross(nt, ex)
    R = side_t / math.sqrt(3.0)
    vs = [ct + R * (np.cos(st + 2 * math.pi * k / 3)[:, None] * ex + np.sin(st + 2 * math.pi * k / 3)[:, None] * ey)
          for k in range(3)]
    Tt = triangle_T(vs[0], vs[1], vs[2])
    ground = helios_patch_T((0.5 * dom, 0.5 * dom, 0.0), (dom, dom))[None, :]
    T, ty, ts, area = _concat([(ground, PATCH, 0, np.array([dom * dom])), (Tp, PATCH, 1, np.full(n_patch, leaf_area)),
                               (Tt, TRIANGLE, 1, np.full(n_tri, leaf_area))])
    return Scene(T, ty, ts, area, {"ground": np.array([0]), "leaves": np.arange(1, n + 1)})


def served_stream(n_requests=2000, rate=50.0, n_scenes=32, n_min=2000, n_max=2000000, seed=0):
    """Request stream of the served configuration: Poisson arrivals at `rate`; each of
    n_scenes scenes is a homogeneous canopy of log-uniform size in [n_min, n_max]
    (patch:triangle 1:1) with LAI U[0.5, 5], its own band set (1-4 of 4 bands), diffuse
    ray count U[50, 400] and seed; each request picks a scene and a sun position (zenith
    U[0, 75] deg, azimuth U[0, 360]) with its direct and diffuse fluxes.  Returns the scene
    sizes and LAIs and the requests (each carrying its scene's bands, rays and seed)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_scenes)).astype(int)
    lais = rng.uniform(0.5, 5.0, n_scenes)
    scene_bands, scene_rays, scene_seed = [], [], []
    for _ in range(n_scenes):
        nb = int(rng.integers(1, 5))
        flags = np.zeros(4, np.uint8)
        flags[rng.choice(4, nb, replace=False)] = 1
        scene_bands.append(flags)
        scene_rays.append(int(rng.integers(50, 401)))
        scene_seed.append(int(rng.integers(1 << 31)))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    reqs = []
    for i in range(n_requests):
        k = int(rng.integers(n_scenes))
        nb = int(scene_bands[k].sum())
        zen = rng.uniform(0.0, 75.0)
        az = rng.uniform(0.0, 360.0)
        reqs.append({"id": i, "scene": k, "arrival": float(arrivals[i]), "bands": scene_bands[k],
                     "sun": sun_direction(zen, az), "direct": rng.uniform(100.0, 600.0, nb).astype(np.float32),
                     "diffuse": rng.uniform(20.0, 150.0, nb).astype(np.float32),
                     "diffuse_rays": scene_rays[k], "seed": scene_seed[k]})
    return sizes, lais, reqs


# leaf optical properties of the four served bands (PAR, NIR, red, green)
SERVED_RHO = np.array([0.08, 0.45, 0.06, 0.12], np.float32)
SERVED_TAU = np.array([0.05, 0.40, 0.04, 0.10], np.float32)
