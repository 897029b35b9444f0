"""Hit-ID comparison against the reference's own CPU ray caster, with every disagreement
classified.  Shared by the CPU test (oracle vs reference, live), the golden-vector script
and the GPU test (device vs the reference's stored hits).

A disagreement between our closest hit (a, t_a) and the reference's (b, t_b) is one of:
- "tmin": the reference hit lies closer than 1e-4, the minimum ray distance of the radiation
  programs (OptiX8DeviceCode.cu:1442, :1621); the reference caster accepts t > 1e-6
  (CollisionDetection_RayTracing.cpp:1562);
- "parallel": the reference caster rejected our triangle as parallel to the ray: its
  Moller-Trumbore determinant e1 . (d x e2) lies below the absolute 1e-5 the caster uses
  (CollisionDetection_RayTracing.cpp:1796-1812), which for a 3 cm leaf means rays within
  about 0.7 degrees of its plane;
- "tie": both hits at the same distance within 1e-6 relative (coincident surfaces: the
  radiation path breaks ties by the smaller index, the caster by its traversal order);
- "grazing": the FP64 intersection of the ray with one of the two primitives lies within
  GRAZE of that primitive's edge (in its canonical unit frame; the caster widens triangles
  by 1e-5 in barycentric terms, CollisionDetection_RayTracing.cpp:1822-1836), or the ray runs
  within GRAZE of parallel to its plane: FP32 rounding decides such hits either way;
- "mismatch": anything else.  The tests require none.
"""
from __future__ import annotations

import numpy as np

TMIN = 1e-4
GRAZE = 2e-5
DET_EPS = 1e-5  # the caster's parallel cutoff on the triangle determinant


def _edge_margin(T, ptype, o, d):
    """(margin, cos) of each ray against the plane of its primitive, FP64: margin > 0
    inside the canonical shape (patch [-0.5,0.5]^2, triangle (0,0),(0,1),(1,1)), < 0
    outside, |margin| = distance to the nearest edge in canonical units."""
    T = np.asarray(T, np.float64).reshape(-1, 4, 4)
    M = T[:, :3, :3]
    c = T[:, :3, 3]
    o = np.asarray(o, np.float64)
    d = np.asarray(d, np.float64)
    A = np.stack([M[:, :, 0], M[:, :, 1], -d], axis=-1)
    nrm = np.cross(M[:, :, 0], M[:, :, 1])
    cosv = np.abs(np.einsum("ij,ij->i", nrm, d)) / np.maximum(np.linalg.norm(nrm, axis=1), 1e-300)
    ok = cosv > 1e-12
    sol = np.zeros((len(o), 3))
    if ok.any():
        sol[ok] = np.linalg.solve(A[ok], (o - c)[ok][..., None])[..., 0]
    u, v = sol[:, 0], sol[:, 1]
    tri = np.asarray(ptype) == 1
    margin = np.where(tri, np.minimum(np.minimum(u, v - u), 1.0 - v), 0.5 - np.maximum(np.abs(u), np.abs(v)))
    margin = np.where(ok, margin, 0.0)
    return margin, cosv


def classify(T, ptype, o, d, ours, t_ours, ref, t_ref):
    """Counts per class over the rays where `ours` (index, -1 miss) differs from `ref`."""
    ours = np.asarray(ours, np.int64)
    ref = np.asarray(ref, np.int64)
    dis = np.nonzero(ours != ref)[0]
    counts = {"rays": int(ours.size), "agree": int(ours.size - dis.size), "tmin": 0, "parallel": 0, "tie": 0,
              "grazing": 0, "mismatch": 0}
    mismatches = []
    if dis.size == 0:
        return counts, mismatches
    T = np.asarray(T).reshape(-1, 16)
    od, dd = np.asarray(o)[dis], np.asarray(d)[dis]
    a, b = ours[dis], ref[dis]
    ta = np.where(a >= 0, np.asarray(t_ours, np.float64)[dis], np.inf)
    tb = np.where(b >= 0, np.asarray(t_ref, np.float64)[dis], np.inf)
    parallel = np.zeros(dis.size, bool)
    tri_a = (a >= 0) & (np.asarray(ptype)[np.maximum(a, 0)] == 1)
    if tri_a.any():
        Ta = T[a[tri_a]].reshape(-1, 4, 4).astype(np.float64)
        e1, e2 = Ta[:, :3, 1], Ta[:, :3, 0] + Ta[:, :3, 1]  # v1 - v0, v2 - v0 of (0,0),(0,1),(1,1)
        det = np.einsum("ij,ij->i", e1, np.cross(dd[tri_a].astype(np.float64), e2))
        parallel[np.nonzero(tri_a)[0]] = np.abs(det) < DET_EPS * 1.01
    graze = np.zeros(dis.size, bool)
    for prim in (a, b):
        has = prim >= 0
        if has.any():
            m, cosv = _edge_margin(T[prim[has]], np.asarray(ptype)[prim[has]], od[has], dd[has])
            graze[np.nonzero(has)[0]] |= (np.abs(m) < GRAZE) | (cosv < GRAZE)
    for k in range(dis.size):
        if b[k] >= 0 and tb[k] < TMIN:
            counts["tmin"] += 1
        elif parallel[k] and (b[k] < 0 or tb[k] > ta[k]):
            counts["parallel"] += 1
        elif np.isfinite(ta[k]) and np.isfinite(tb[k]) and abs(ta[k] - tb[k]) <= 1e-6 * max(ta[k], tb[k]):
            counts["tie"] += 1
        elif graze[k]:
            counts["grazing"] += 1
        else:
            counts["mismatch"] += 1
            mismatches.append((int(dis[k]), int(a[k]), float(ta[k]), int(b[k]), float(tb[k])))
    return counts, mismatches


def free_space_rays(lo, hi, n, seed):
    """n rays with origins uniform in the box [lo, hi] and directions uniform on the sphere."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    o = (lo + (hi - lo) * rng.uniform(size=(n, 3))).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    return o, d
