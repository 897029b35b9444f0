// hrt_oracle.cpp -- CPU FP64 oracle for the Helios radiation-transfer hot path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product (helios_gb300/) links, loads
// or calls this file; only tests/, __graft_entry__.smoke() (as the checker) and
// bench.py's cpu_baseline / --impl reference legs use it.
//
// What it restates (reference = PlantSimulationLab/Helios, plugin "radiation"):
//   * ray generation          src/optix8/OptiX8DeviceCode.cu:1210-1465 (__raygen__direct)
//                              src/optix8/OptiX8DeviceCode.cu:1471-1658 (__raygen__diffuse)
//   * primitive intersection   src/optix8/OptiX8DeviceCode.cu:320-490  (__intersection__patch,
//                              kept as the "reference formula" mode) plus the watertight
//                              test (Woop, Benthin, Wald, JCGT 2013) used by the GPU build
//   * energy deposition        src/optix8/OptiX8DeviceCode.cu:514-596  (__miss__direct)
//                              src/optix8/OptiX8DeviceCode.cu:598-671  (__miss__diffuse)
//                              src/optix8/OptiX8DeviceCode.cu:930-1001 (__closesthit__diffuse)
//                              src/optix8/OptiX8DeviceCode.cu:148-164  (sky distribution)
//   * buffer bookkeeping       src/backends/OptiX8Backend.cpp:1168-1250
//   * pass orchestration       src/RadiationModel.cpp:3470-4663 (runBand)
//   * emission source term     src/RadiationModel.cpp:4041-4137 (sigma*eps*T^4)
//
// Arithmetic contract: every FP32 operation on the geometric path (ray generation,
// bounding boxes, Morton codes, slab and primitive tests) is written as a plain
// sequence of IEEE-754 single-precision +, -, *, / and sqrt, compiled with
// -ffp-contract=off.  The CUDA kernels compile the same sequences with
// --fmad=false, so both sides produce bit-identical rays, BVHs and hit IDs.
// Energy sums are FP64 here (the "FP64 oracle").
//
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), keyed by
// (seed, pass) with counter (ray, primitive, face|source<<1, 0).  The reference
// uses TEA16 + LCG seeded from the wall clock (RadiationModel.cpp:3961), so its
// ray sets are not reproducible; parity with the reference is statistical.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- vectors ---
struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 vsub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 vadd(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 vscale(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline float vdot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 vcross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline V3 vnormalize(V3 a) {
    float l = std::sqrt(vdot(a, a));
    return v3(a.x / l, a.y / l, a.z / l);
}
inline float vget(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

// T . (px, py, 0, 1) for a row-major 4x4 transform, fixed evaluation order.
inline V3 xform(const float *T, float px, float py) {
    return v3((T[0] * px + T[1] * py) + T[3], (T[4] * px + T[5] * py) + T[7],
              (T[8] * px + T[9] * py) + T[11]);
}

// ---------------------------------------------------------------- Philox ---
struct U4 {
    uint32_t v[4];
};
inline U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
    }
    return U4{{c0, c1, c2, c3}};
}
inline float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// ------------------------------------------------- reference random numbers ---
// Statistical parity only (orc_set_rng(1)): the reference seeds each ray's stream with
// TEA, 16 rounds (Wheeler & Needham, FSE 1994; the reference's keys), of (ray index,
// launch seed) and draws 24-bit uniforms from a linear congruential generator with the
// Numerical Recipes constants (OptiX8DeviceCode.cu:29-49; per-ray seeding :1232, :1497).
// The four uniforms of one call are four consecutive draws of that stream, consumed in the
// reference's order (direction jitter, then origin).  The reference's launch seed comes from
// the wall clock (RadiationModel.cpp:3961); here it is TEA of (seed, pass, counter words),
// and the ray index is TEA-mixed from (ray, primitive).
int g_rng_mode = 0;  // 0 Philox (the product's stream), 1 reference TEA + LCG

inline uint32_t tea16(uint32_t a, uint32_t b) {
    uint32_t sum = 0;
    for (int round = 0; round < 16; ++round) {
        sum += 0x9E3779B9u;
        a += ((b << 4) + 0xA341316Cu) ^ (b + sum) ^ ((b >> 5) + 0xC8013EA4u);
        b += ((a << 4) + 0xAD90777Du) ^ (a + sum) ^ ((a >> 5) + 0x7E95761Eu);
    }
    return a;
}

inline uint32_t lcg24(uint32_t *state) {
    *state = 1664525u * *state + 1013904223u;
    return *state & 0x00FFFFFFu;
}

// Four uniforms for counter (c0 ray, c1 primitive, c2, c3) and key (k0 seed, k1 pass).
inline U4 draw(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
    if (g_rng_mode == 0) return philox(c0, c1, c2, c3, k0, k1);
    const uint32_t launch = tea16(tea16(k0, k1), tea16(c2, c3));
    uint32_t st = tea16(tea16(c0, c1), launch);
    U4 u;
    for (int k = 0; k < 4; ++k) u.v[k] = lcg24(&st) << 8;  // u01 keeps the top 24 bits
    return u;
}

// cos(2*pi*u), sin(2*pi*u) for u in [0,1): quadrant/octant reduction and
// Taylor polynomials on [0, pi/4] (coefficients are 1/k!), evaluated in a fixed order.
inline void sincos2pi(float u, float *c_out, float *s_out) {
    float x = u * 4.0f;
    int q = (int)x;
    float f = x - (float)q;
    bool swap = f > 0.5f;
    float g = swap ? (1.0f - f) : f;
    float a = g * 1.57079632679489662f;
    float a2 = a * a;
    float s = a + a * a2 * (-1.66666666666666667e-1f +
                            a2 * (8.33333333333333333e-3f +
                                  a2 * (-1.98412698412698413e-4f + a2 * 2.75573192239858907e-6f)));
    float c = 1.0f + a2 * (-0.5f + a2 * (4.16666666666666667e-2f +
                                         a2 * (-1.38888888888888889e-3f +
                                               a2 * (2.48015873015873016e-5f +
                                                     a2 * -2.75573192239858907e-7f))));
    float c0 = swap ? s : c;
    float s0 = swap ? c : s;
    q &= 3;
    if (q == 0) {
        *c_out = c0;
        *s_out = s0;
    } else if (q == 1) {
        *c_out = -s0;
        *s_out = c0;
    } else if (q == 2) {
        *c_out = -c0;
        *s_out = -s0;
    } else {
        *c_out = s0;
        *s_out = -c0;
    }
}

// Natural logarithm of x in (0, 1] (the free-path draw of the voxel medium), in plain
// IEEE single-precision steps so host and device agree bit for bit: x = m * 2^e with
// m in [sqrt(1/2), sqrt(2)), then ln m = 2 atanh(z), z = (m - 1) / (m + 1), by its
// Taylor series to z^9 (|z| <= 0.172, truncation below 1e-9).
inline float ln_unit(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    int e = (int)((b >> 23) & 0xFFu) - 127;
    uint32_t mb = (b & 0x7FFFFFu) | 0x3F800000u;
    float m;
    std::memcpy(&m, &mb, 4);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e = e + 1;
    }
    float z = (m - 1.0f) / (m + 1.0f);
    float z2 = z * z;
    float s = 1.0f + z2 * (0.333333333f + z2 * (0.2f + z2 * (0.142857143f + z2 * 0.111111111f)));
    return (float)e * 0.693147181f + 2.0f * z * s;
}

// Concentric square-to-disk map (Shirley & Chiu, "A Low Distortion Map Between Disk and
// Square", JGT 1997) of (u, v) in [0,1)^2 to the unit disk; the angle is evaluated as a
// fraction of a turn by sincos2pi.
inline void concentric(float u, float v, float *x, float *y) {
    float sx = -1.0f + 2.0f * u, sy = -1.0f + 2.0f * v;
    float r, ph;  // ph in units of pi/4
    if (sx > -sy) {
        if (sx > sy) { r = sx; ph = sy / sx; }
        else { r = sy; ph = 2.0f - sx / sy; }
    } else {
        if (sx < sy) { r = -sx; ph = 4.0f + sy / sx; }
        else { r = -sy; ph = (sy != 0.f) ? 6.0f - sx / sy : 0.f; }
    }
    float frac = ph * 0.125f;
    if (frac < 0.f) frac = frac + 1.0f;
    float c, s;
    sincos2pi(frac, &c, &s);
    *x = r * c;
    *y = r * s;
}

// Orthonormal basis around unit n (Duff, Burgess, Christensen, Hery, Kensler,
// Liani, Villemin: "Building an Orthonormal Basis, Revisited", JCGT 6(1), 2017).
inline void onb(V3 n, V3 *t1, V3 *t2) {
    float sign = std::copysign(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    *t1 = v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    *t2 = v3(b, sign + n.y * n.y * a, -n.y);
}

// ---------------------------------------------------------------- records ---
// Primitive types (RayTracingTypes.h:45): 0 patch, 1 triangle, 2 disk, 3 tile, 4 voxel, 5 bbox face.
enum { PT_PATCH = 0, PT_TRI = 1, PT_DISK = 2, PT_TILE = 3, PT_VOXEL = 4, PT_BBOX = 5 };

struct Rec {        // intersection record, one per primitive
    V3 p[4];        // patch/bbox: 4 corners; triangle: v0,v1,v2; disk: centre, normal(unit), (r,0,0)
    int type;       // voxel: p[0]=lo, p[1]=hi
    float k;        // voxel: extinction coefficient G * LAD (1/m), G = 0.5
};
struct RGen {       // ray-origin sampling record
    V3 P, A, B, N;  // point = P + u*A + v*B ; N = unit normal (voxel: N = third box edge C)
};

// Projection coefficient of the voxel medium's leaves: G = 0.5 (spherical leaf angles).
constexpr float kVoxelG = 0.5f;

Rec make_rec(const float *T, int type, float lad) {
    Rec r{};
    r.type = type;
    if (type == PT_TRI) {
        r.p[0] = xform(T, 0.f, 0.f);
        r.p[1] = xform(T, 0.f, 1.f);
        r.p[2] = xform(T, 1.f, 1.f);
        r.p[3] = r.p[2];
    } else if (type == PT_DISK) {
        // unit disk in the canonical xy plane; T scales it (OptiX 6 primitiveIntersection.cu:236-300)
        r.p[0] = xform(T, 0.f, 0.f);
        V3 ax = v3(T[0], T[4], T[8]);
        V3 ay = v3(T[1], T[5], T[9]);
        r.p[1] = vnormalize(vcross(ax, ay));
        r.p[2] = v3(std::sqrt(vdot(ax, ax)), 0.f, 0.f);
        r.p[3] = r.p[0];
    } else if (type == PT_VOXEL) {
        // axis-aligned box: canonical [-0.5,0.5]^3 scaled/translated by T (diagonal part only)
        V3 c = v3(T[3], T[7], T[11]);
        V3 h = v3(std::fabs(T[0]) * 0.5f, std::fabs(T[5]) * 0.5f, std::fabs(T[10]) * 0.5f);
        r.p[0] = vsub(c, h);
        r.p[1] = vadd(c, h);
        r.p[2] = r.p[0];
        r.p[3] = r.p[1];
        r.k = kVoxelG * lad;
    } else {  // patch, tile
        r.type = PT_PATCH;
        r.p[0] = xform(T, -0.5f, -0.5f);
        r.p[1] = xform(T, 0.5f, -0.5f);
        r.p[2] = xform(T, 0.5f, 0.5f);
        r.p[3] = xform(T, -0.5f, 0.5f);
    }
    return r;
}

RGen make_rgen(const float *T, int type) {
    RGen g{};
    g.A = v3(T[0], T[4], T[8]);
    g.B = v3(T[1], T[5], T[9]);
    if (type == PT_TRI) {
        g.P = v3(T[3], T[7], T[11]);
        g.N = vnormalize(vcross(g.B, g.A));  // = normalize(cross(v1-v0, v2-v0))
    } else if (type == PT_DISK) {
        g.P = v3(T[3], T[7], T[11]);         // centre; the unit disk spans A and B
        g.N = vnormalize(vcross(g.A, g.B));
    } else if (type == PT_VOXEL) {
        g.N = v3(T[2], T[6], T[10]);         // third edge of the box
        g.P = v3(((T[0] * -0.5f + T[1] * -0.5f) + T[2] * -0.5f) + T[3],
                 ((T[4] * -0.5f + T[5] * -0.5f) + T[6] * -0.5f) + T[7],
                 ((T[8] * -0.5f + T[9] * -0.5f) + T[10] * -0.5f) + T[11]);
    } else {
        g.P = xform(T, -0.5f, -0.5f);
        g.N = vnormalize(vcross(g.A, g.B));
    }
    return g;
}

// Surface area of a primitive (leaf area for a voxel: LAD x volume), in FP64 from the
// FP32 transform; it weights the scattering residual.
double prim_area(const float *T, int type, float lad) {
    double ax = T[0], ay = T[4], az = T[8], bx = T[1], by = T[5], bz = T[9];
    if (type == PT_VOXEL) {
        double cx = T[2], cy = T[6], cz = T[10];
        double det = ax * (by * cz - bz * cy) - bx * (ay * cz - az * cy) + cx * (ay * bz - az * by);
        return (double)lad * std::fabs(det);
    }
    double x = ay * bz - az * by, y = az * bx - ax * bz, z = ax * by - ay * bx;
    double a = std::sqrt(x * x + y * y + z * z);
    if (type == PT_TRI) return 0.5 * a;
    if (type == PT_DISK) return M_PI * a;
    return a;
}

void rec_bounds(const Rec &r, V3 *lo, V3 *hi) {
    if (r.type == PT_DISK) {
        V3 c = r.p[0], n = r.p[1];
        float rad = r.p[2].x;
        // extent of a disk of radius rad with normal n along axis k: rad*sqrt(1-n_k^2)
        float ex = rad * std::sqrt(std::fmax(0.f, 1.0f - n.x * n.x));
        float ey = rad * std::sqrt(std::fmax(0.f, 1.0f - n.y * n.y));
        float ez = rad * std::sqrt(std::fmax(0.f, 1.0f - n.z * n.z));
        *lo = v3(c.x - ex, c.y - ey, c.z - ez);
        *hi = v3(c.x + ex, c.y + ey, c.z + ez);
        return;
    }
    int nv = (r.type == PT_TRI) ? 3 : (r.type == PT_VOXEL ? 2 : 4);
    V3 a = r.p[0], b = r.p[0];
    for (int i = 1; i < nv; ++i) {
        a = v3(std::fmin(a.x, r.p[i].x), std::fmin(a.y, r.p[i].y), std::fmin(a.z, r.p[i].z));
        b = v3(std::fmax(b.x, r.p[i].x), std::fmax(b.y, r.p[i].y), std::fmax(b.z, r.p[i].z));
    }
    *lo = a;
    *hi = b;
}

// ---------------------------------------------------------------- rays -----
// Philox counter words c0..c2 and key of a ray's voxel free-path draws; the draw for
// voxel v is philox(c0, c1, c2 | wrap << 16, v + 1; k0, k1), so it depends on the ray's
// identity and the periodic wrap only, never on traversal order or launch batching.
struct VoxKey {
    uint32_t c0, c1, c2, k0, k1;
};
struct Ray {
    V3 o, d;
    float tmin, tmax;
    VoxKey key;
};
struct Hit {
    float t;
    int32_t prim;  // original primitive index, -1 = miss
    int32_t face;  // 1 = ray hit the top (front) face, 0 = bottom
};

// Per-ray precomputation for the watertight test.
struct WT {
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
inline WT wt_setup(V3 d) {
    WT w;
    float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    w.kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    w.kx = (w.kz + 1) % 3;
    w.ky = (w.kx + 1) % 3;
    if (vget(d, w.kz) < 0.f) std::swap(w.kx, w.ky);
    float dz = vget(d, w.kz);
    w.Sx = vget(d, w.kx) / dz;
    w.Sy = vget(d, w.ky) / dz;
    w.Sz = 1.0f / dz;
    return w;
}

// 2-D edge function e(P,Q) = Px*Qy - Py*Qx with an FP64 recompute when it is exactly 0.
inline float edgef(float px, float py, float qx, float qy) {
    float e = px * qy - py * qx;
    if (e == 0.f) e = (float)((double)px * (double)qy - (double)py * (double)qx);
    return e;
}

// Watertight polygon test (triangle: n=3, planar convex quad: n=4).  Returns t or -1.
// face: 1 when the ray arrives on the side the geometric normal points to is *not*
// the side it comes from, i.e. dot(d, n) < 0 (top face), matching the reference's
// face attribute (OptiX8DeviceCode.cu:421,485).
inline bool poly_hit(const WT &w, const Ray &ray, const V3 *v, int n, float tmax, float *t_out,
                     int *face_out) {
    float px[4], py[4], pz[4];
    for (int i = 0; i < n; ++i) {
        V3 a = vsub(v[i], ray.o);
        float az = vget(a, w.kz);
        px[i] = vget(a, w.kx) - w.Sx * az;
        py[i] = vget(a, w.ky) - w.Sy * az;
        pz[i] = w.Sz * az;
    }
    float e[4];
    for (int i = 0; i < n; ++i) {
        int j = (i + 1 == n) ? 0 : i + 1;
        e[i] = edgef(px[i], py[i], px[j], py[j]);
    }
    bool anyneg = false, anypos = false;
    for (int i = 0; i < n; ++i) {
        anyneg = anyneg || (e[i] < 0.f);
        anypos = anypos || (e[i] > 0.f);
    }
    if (anyneg && anypos) return false;
    // barycentric weights of triangle (v0, v1, v2): w0 = e(v1,v2), w1 = e(v2,v0), w2 = e(v0,v1)
    float e20 = (n == 3) ? e[2] : edgef(px[2], py[2], px[0], py[0]);
    float det = (e[1] + e20) + e[0];
    if (det == 0.f) return false;
    float T = (e[1] * pz[0] + e20 * pz[1]) + e[0] * pz[2];
    float t = T / det;
    if (!(t >= ray.tmin) || !(t <= tmax)) return false;
    *t_out = t;
    // det < 0 <=> dot(d, n) < 0 for n = (v1-v0) x (v2-v0): the ray meets the top face
    *face_out = (det < 0.f) ? 1 : 0;
    return true;
}

// Disk (OptiX 6 primitiveIntersection.cu:236-300 semantics: plane hit inside radius).
inline bool disk_hit(const Ray &ray, const Rec &r, float tmax, float *t_out, int *face_out) {
    V3 c = r.p[0], n = r.p[1];
    float rad = r.p[2].x;
    float nd = vdot(ray.d, n);
    if (nd == 0.f) return false;
    float t = vdot(vsub(c, ray.o), n) / nd;
    if (!(t >= ray.tmin) || !(t <= tmax)) return false;
    V3 h = vsub(vadd(ray.o, vscale(ray.d, t)), c);
    if (vdot(h, h) > rad * rad) return false;
    *t_out = t;
    *face_out = (nd < 0.f) ? 1 : 0;
    return true;
}

// Slab test against an axis-aligned box; used for voxels and BVH nodes.
inline bool slab(const V3 &o, const V3 &inv, V3 lo, V3 hi, float tmin, float tmax, float *tnear) {
    float t0x = (lo.x - o.x) * inv.x, t1x = (hi.x - o.x) * inv.x;
    float t0y = (lo.y - o.y) * inv.y, t1y = (hi.y - o.y) * inv.y;
    float t0z = (lo.z - o.z) * inv.z, t1z = (hi.z - o.z) * inv.z;
    float tn = std::fmax(std::fmax(std::fmin(t0x, t1x), std::fmin(t0y, t1y)),
                         std::fmax(std::fmin(t0z, t1z), tmin));
    float tf = std::fmin(std::fmin(std::fmax(t0x, t1x), std::fmax(t0y, t1y)),
                         std::fmin(std::fmax(t0z, t1z), tmax));
    *tnear = tn;
    return tn <= tf;
}
// BVH node boxes: t = lo * inv - o * inv with one fused multiply-add per plane.
inline bool slab_node(const V3 &ooi, const V3 &inv, V3 lo, V3 hi, float tmin, float tmax, float *tnear) {
    float t0x = std::fma(lo.x, inv.x, -ooi.x), t1x = std::fma(hi.x, inv.x, -ooi.x);
    float t0y = std::fma(lo.y, inv.y, -ooi.y), t1y = std::fma(hi.y, inv.y, -ooi.y);
    float t0z = std::fma(lo.z, inv.z, -ooi.z), t1z = std::fma(hi.z, inv.z, -ooi.z);
    float tn = std::fmax(std::fmax(std::fmin(t0x, t1x), std::fmin(t0y, t1y)),
                         std::fmax(std::fmin(t0z, t1z), tmin));
    float tf = std::fmin(std::fmin(std::fmax(t0x, t1x), std::fmax(t0y, t1y)),
                         std::fmin(std::fmax(t0z, t1z), tmax));
    *tnear = tn;
    return tn <= tf;
}
inline float safe_inv(float d) {
    if (std::fabs(d) < 1e-30f) d = std::copysign(1e-30f, d);
    return 1.0f / d;
}

// Voxel: a turbid medium of leaf area density LAD with extinction k = G * LAD.  The
// reference has no voxel physics (its OptiX 6 voxel absorption is commented out,
// rayHit.cu:278-290), so this one is defined here: the ray's path through the box from
// max(entry, tmin) to the exit is intercepted at the free path s = -ln(xi) / k, xi
// uniform in (0, 1] drawn per (ray, voxel, wrap).  A ray starting inside the box crosses
// the rest of it (the reference's "inside origin: no hit" rule, primitiveIntersection.cu:
// 330-374, would let a voxel's own leaves see through it).  The hit is always the top face.
inline bool voxel_hit(const Ray &ray, const V3 &inv, const Rec &r, uint32_t vid, float tmax, float *t_out,
                      int *face_out) {
    if (!(r.k > 0.f)) return false;
    V3 lo = r.p[0], hi = r.p[1], o = ray.o;
    float t0x = (lo.x - o.x) * inv.x, t1x = (hi.x - o.x) * inv.x;
    float t0y = (lo.y - o.y) * inv.y, t1y = (hi.y - o.y) * inv.y;
    float t0z = (lo.z - o.z) * inv.z, t1z = (hi.z - o.z) * inv.z;
    float tn = std::fmax(std::fmax(std::fmin(t0x, t1x), std::fmin(t0y, t1y)),
                         std::fmax(std::fmin(t0z, t1z), ray.tmin));
    float tf = std::fmin(std::fmin(std::fmax(t0x, t1x), std::fmax(t0y, t1y)), std::fmax(t0z, t1z));
    if (!(tn < tf)) return false;
    U4 u = draw(ray.key.c0, ray.key.c1, ray.key.c2, vid + 1u, ray.key.k0, ray.key.k1);
    float s = -ln_unit(1.0f - u01(u.v[0])) / r.k;
    float t = tn + s;
    if (!(t < tf) || !(t <= tmax)) return false;
    *t_out = t;
    *face_out = 1;
    return true;
}

// Texture masks (OptiX8DeviceCode.cu:173-187, 397-416, 457-476): a masked patch or triangle
// is hit only where its mask texel is opaque.  (u, v) follow the reference: patches from
// the local coordinates of the hit point, triangles from the Cramer barycentrics; custom
// per-primitive UVs are mapped linearly (patches) or barycentrically (triangles).
struct Masks {
    std::vector<int32_t> id, uv_id, size;  // [n], [n], [nm*2]
    std::vector<float> uv;                 // [n*8]: corners (u,v) 0..3
    std::vector<uint32_t> offset;          // [nm]
    std::vector<uint8_t> data;
    const float *T = nullptr;              // transforms of the scene
};

inline bool mask_opaque(const Masks &m, int id, float u, float v) {
    const int w = m.size[2 * id], h = m.size[2 * id + 1];
    int ix = (int)std::floor((float)(w - 1) * u);
    int iy = (int)std::floor((float)(h - 1) * (1.0f - v));
    ix = ix < 0 ? 0 : (ix > w - 1 ? w - 1 : ix);
    iy = iy < 0 ? 0 : (iy > h - 1 ? h - 1 : iy);
    return m.data[m.offset[id] + (uint32_t)(iy * w + ix)] != 0;
}

// texture (u, v) of patch p at local coordinates (lu, lv) in [-0.5, 0.5]^2
inline void patch_uv(const Masks &m, int p, float lu, float lv, float *uu, float *vv) {
    if (m.uv_id[p] >= 0) {
        const float *q = &m.uv[8 * (size_t)p];
        *uu = q[0] + (lu + 0.5f) * (q[2] - q[0]);
        *vv = q[1] + (lv + 0.5f) * (q[5] - q[1]);
    } else {
        *uu = lu + 0.5f;
        *vv = lv + 0.5f;
    }
}

// texture (u, v) of triangle p at barycentrics beta (vertex 1) and gamma (vertex 2)
inline void tri_uv(const Masks &m, int p, float beta, float gamma, float *uu, float *vv) {
    if (m.uv_id[p] >= 0) {
        const float *q = &m.uv[8 * (size_t)p];
        *uu = (q[0] + beta * (q[2] - q[0])) + gamma * (q[4] - q[0]);
        *vv = 1.0f - ((q[1] + beta * (q[3] - q[1])) + gamma * (q[5] - q[1]));
    } else {
        *uu = beta + gamma;
        *vv = gamma;
    }
}

// Is the geometric hit at distance t on masked primitive p on an opaque texel?
inline bool mask_hit_opaque(const Masks &m, int p, int type, const Ray &ray, float t) {
    const float *T = m.T + 16 * (size_t)p;
    V3 o = ray.o, d = ray.d;
    float uu, vv;
    if (type == PT_TRI) {
        V3 v0 = v3(T[3], T[7], T[11]);
        V3 v1 = xform(T, 0.f, 1.f), v2 = xform(T, 1.f, 1.f);
        float a = v0.x - v1.x, b = v0.x - v2.x, c = d.x, dd = v0.x - o.x;
        float e = v0.y - v1.y, f = v0.y - v2.y, g = d.y, h = v0.y - o.y;
        float i = v0.z - v1.z, j = v0.z - v2.z, k = d.z, l = v0.z - o.z;
        float mm = f * k - g * j, nn = h * k - g * l, pp = f * l - h * j;
        float q = g * i - e * k, sq = e * j - f * i;
        float den = a * mm + b * q + c * sq;
        if (den == 0.f) return true;
        float iv = 1.f / den;
        float beta = (dd * mm - b * nn - c * pp) * iv;
        float r = e * l - h * i;
        float gamma = (a * nn + dd * q + c * r) * iv;
        tri_uv(m, p, beta, gamma, &uu, &vv);
    } else {
        V3 hl = vsub(vadd(o, vscale(d, t)), v3(T[3], T[7], T[11]));
        V3 lx = v3(T[0], T[4], T[8]), ly = v3(T[1], T[5], T[9]);
        float lu = vdot(hl, lx) / vdot(lx, lx), lv = vdot(hl, ly) / vdot(ly, ly);
        patch_uv(m, p, lu, lv, &uu, &vv);
    }
    return mask_opaque(m, m.id[p], uu, vv);
}

inline bool prim_hit(const WT &w, const Ray &ray, const V3 &inv, const Rec &r, uint32_t id, float tmax,
                     float *t, int *face, const Masks *mk = nullptr) {
    switch (r.type) {
        case PT_TRI:
            if (!poly_hit(w, ray, r.p, 3, tmax, t, face)) return false;
            return !(mk && mk->id[id] >= 0) || mask_hit_opaque(*mk, (int)id, PT_TRI, ray, *t);
        case PT_PATCH:
            if (!poly_hit(w, ray, r.p, 4, tmax, t, face)) return false;
            return !(mk && mk->id[id] >= 0) || mask_hit_opaque(*mk, (int)id, PT_PATCH, ray, *t);
        case PT_BBOX:
            return poly_hit(w, ray, r.p, 4, tmax, t, face);
        case PT_DISK:
            return disk_hit(ray, r, tmax, t, face);
        case PT_VOXEL:
            return voxel_hit(ray, inv, r, id, tmax, t, face);
    }
    return false;
}

// Reference intersection formulas, restated from OptiX8DeviceCode.cu:369-489
// (patch: plane + local (u,v) in [-0.5,0.5]^2; triangle: Shirley/Cramer form).
inline bool prim_hit_reference(const Ray &ray, const float *T, int type, float tmax, float *t_out,
                               int *face_out) {
    V3 o = ray.o, d = ray.d;
    if (type == PT_PATCH || type == PT_TILE) {
        V3 n = v3(T[2], T[6], T[10]);
        float nd = vdot(d, n);
        if (std::fabs(nd) < 1e-8f) return false;
        V3 c = v3(T[3], T[7], T[11]);
        float t = vdot(vsub(c, o), n) / nd;
        if (t < ray.tmin || t > tmax) return false;
        V3 hl = vsub(vadd(o, vscale(d, t)), c);
        V3 lx = v3(T[0], T[4], T[8]), ly = v3(T[1], T[5], T[9]);
        float lx2 = vdot(lx, lx), ly2 = vdot(ly, ly);
        if (lx2 < 1e-12f || ly2 < 1e-12f) return false;
        float u = vdot(hl, lx) / lx2, v = vdot(hl, ly) / ly2;
        if (u < -0.5f || u > 0.5f || v < -0.5f || v > 0.5f) return false;
        *t_out = t;
        *face_out = (nd < 0.f) ? 1 : 0;
        return true;
    }
    if (type != PT_TRI) return false;
    V3 v0 = v3(T[3], T[7], T[11]);
    V3 v1 = v3(T[1] + T[3], T[5] + T[7], T[9] + T[11]);
    V3 v2 = v3(T[0] + T[1] + T[3], T[4] + T[5] + T[7], T[8] + T[9] + T[11]);
    float a = v0.x - v1.x, b = v0.x - v2.x, c = d.x, dd = v0.x - o.x;
    float e = v0.y - v1.y, f = v0.y - v2.y, g = d.y, h = v0.y - o.y;
    float i = v0.z - v1.z, j = v0.z - v2.z, k = d.z, l = v0.z - o.z;
    float m = f * k - g * j, nn = h * k - g * l, p = f * l - h * j;
    float q = g * i - e * k, s = e * j - f * i;
    float den = a * m + b * q + c * s;
    if (std::fabs(den) < 1e-12f) return false;
    float inv = 1.f / den;
    float beta = (dd * m - b * nn - c * p) * inv;
    if (beta < 0.f) return false;
    float r = e * l - h * i;
    float gamma = (a * nn + dd * q + c * r) * inv;
    if (gamma < 0.f || beta + gamma > 1.f) return false;
    float t = (a * p - b * r + dd * s) * inv;
    if (t < ray.tmin || t > tmax) return false;
    V3 nrm = vcross(vsub(v1, v0), vsub(v2, v0));
    *t_out = t;
    *face_out = (vdot(d, nrm) < 0.f) ? 1 : 0;
    return true;
}

// ---------------------------------------------------------------- LBVH -----
inline uint64_t expand21(uint32_t v) {
    uint64_t x = v & 0x1FFFFFu;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}
inline uint32_t quant21(float c, float lo, float scale) {
    float q = (c - lo) * scale;
    if (!(q > 0.f)) q = 0.f;
    if (q > 2097151.0f) q = 2097151.0f;
    return (uint32_t)q;
}
inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }
inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

// Leaf bounds padding: each face moves out by (|x| + extent) * 2^-20 so that the
// FP32 slab test never rejects a box holding an accepted primitive hit.
inline float pad_lo(float x, float ext) { return x - (std::fabs(x) + ext) * 9.5367431640625e-07f; }
inline float pad_hi(float x, float ext) { return x + (std::fabs(x) + ext) * 9.5367431640625e-07f; }

struct Node {       // BVH2 node: both child boxes + child references
    float b[12];    // c0.lo.xyz, c0.hi.xyz, c1.lo.xyz, c1.hi.xyz
    int32_t c[2];   // >= 0: internal node; < 0: ~leaf (sorted primitive slot)
};

struct Scene {
    int n = 0;
    std::vector<float> T;
    std::vector<uint32_t> type;
    std::vector<int8_t> twosided;
    std::vector<Rec> rec;       // original order
    std::vector<RGen> rgen;     // original order
    std::vector<double> area;   // original order (voxels: leaf area)
    Masks masks;                // texture masks (empty: none)
    const Masks *mk() const { return masks.id.empty() ? nullptr : &masks; }
    // BVH
    std::vector<uint64_t> codes;    // sorted Morton codes
    std::vector<uint32_t> perm;     // sorted slot -> original primitive
    std::vector<Node> nodes;        // n-1 internal nodes (1 for n == 1)
    std::vector<float> leaf_lo, leaf_hi;  // padded leaf boxes, sorted order (3 each)
    float scene_lo[3], scene_hi[3], extent;
    // periodic boundary (bbox faces appended after the n real primitives)
    int nbbox = 0;
    float periodic[2] = {0, 0};
    std::vector<Rec> bbox;
};

void build_bvh(Scene &s) {
    const int n = s.n;
    std::vector<V3> lo(n), hi(n), cen(n);
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float blo[3] = {INFINITY, INFINITY, INFINITY}, bhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < n; ++i) {
        rec_bounds(s.rec[i], &lo[i], &hi[i]);
        cen[i] = v3((lo[i].x + hi[i].x) * 0.5f, (lo[i].y + hi[i].y) * 0.5f, (lo[i].z + hi[i].z) * 0.5f);
        for (int k = 0; k < 3; ++k) {
            clo[k] = std::fmin(clo[k], vget(cen[i], k));
            chi[k] = std::fmax(chi[k], vget(cen[i], k));
            blo[k] = std::fmin(blo[k], vget(lo[i], k));
            bhi[k] = std::fmax(bhi[k], vget(hi[i], k));
        }
    }
    float ext = 0.f;
    for (int k = 0; k < 3; ++k) {
        s.scene_lo[k] = blo[k];
        s.scene_hi[k] = bhi[k];
        ext = std::fmax(ext, bhi[k] - blo[k]);
    }
    s.extent = ext;
    float scale[3];
    for (int k = 0; k < 3; ++k) {
        float e = chi[k] - clo[k];
        scale[k] = (e > 0.f) ? (2097152.0f / e) : 0.f;
    }
    std::vector<std::pair<uint64_t, uint32_t>> kv(n);
    for (int i = 0; i < n; ++i) {
        uint64_t code = (expand21(quant21(cen[i].x, clo[0], scale[0])) << 2) |
                        (expand21(quant21(cen[i].y, clo[1], scale[1])) << 1) |
                        expand21(quant21(cen[i].z, clo[2], scale[2]));
        if (s.rec[i].type == PT_VOXEL) code |= 1ull << 63;  // voxels: their own subtree
        kv[i] = {code, (uint32_t)i};
    }
    std::sort(kv.begin(), kv.end());
    s.codes.resize(n);
    s.perm.resize(n);
    s.leaf_lo.resize(3 * (size_t)n);
    s.leaf_hi.resize(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        s.codes[i] = kv[i].first;
        s.perm[i] = kv[i].second;
        V3 a = lo[kv[i].second], b = hi[kv[i].second];
        s.leaf_lo[3 * i + 0] = pad_lo(a.x, ext);
        s.leaf_lo[3 * i + 1] = pad_lo(a.y, ext);
        s.leaf_lo[3 * i + 2] = pad_lo(a.z, ext);
        s.leaf_hi[3 * i + 0] = pad_hi(b.x, ext);
        s.leaf_hi[3 * i + 1] = pad_hi(b.y, ext);
        s.leaf_hi[3 * i + 2] = pad_hi(b.z, ext);
    }
    // Karras 2012 ("Maximizing parallelism in the construction of BVHs, octrees
    // and k-d trees", HPG 2012) hierarchy over the sorted codes.
    const int ni = std::max(n - 1, 1);
    s.nodes.assign(ni, Node{});
    std::vector<int32_t> parent_internal(ni, -1), parent_leaf(n, -1);
    auto delta = [&](int i, int j) -> int {
        if (j < 0 || j > n - 1) return -1;
        uint64_t a = s.codes[i], b = s.codes[j];
        if (a == b) return 64 + clz32((uint32_t)i ^ (uint32_t)j);
        return clz64(a ^ b);
    };
    if (n == 1) {
        Node &nd = s.nodes[0];
        nd.c[0] = ~0;
        nd.c[1] = ~0x7FFFFFFF;  // empty sentinel (box never hit)
        parent_leaf[0] = 0;
    } else {
        for (int i = 0; i < n - 1; ++i) {
            int dsgn = (delta(i, i + 1) - delta(i, i - 1)) >= 0 ? 1 : -1;
            int dmin = delta(i, i - dsgn);
            int lmax = 2;
            while (delta(i, i + lmax * dsgn) > dmin) lmax *= 2;
            int l = 0;
            for (int t = lmax / 2; t >= 1; t /= 2)
                if (delta(i, i + (l + t) * dsgn) > dmin) l += t;
            int j = i + l * dsgn;
            int dnode = delta(i, j);
            int sp = 0;
            int t = l;
            do {
                t = (t + 1) >> 1;
                if (delta(i, i + (sp + t) * dsgn) > dnode) sp += t;
            } while (t > 1);
            int gamma = i + sp * dsgn + std::min(dsgn, 0);
            int lo_i = std::min(i, j), hi_i = std::max(i, j);
            Node &nd = s.nodes[i];
            if (lo_i == gamma) {
                nd.c[0] = ~gamma;
                parent_leaf[gamma] = i;
            } else {
                nd.c[0] = gamma;
                parent_internal[gamma] = i;
            }
            if (hi_i == gamma + 1) {
                nd.c[1] = ~(gamma + 1);
                parent_leaf[gamma + 1] = i;
            } else {
                nd.c[1] = gamma + 1;
                parent_internal[gamma + 1] = i;
            }
        }
    }
    // Bottom-up refit: a node's box is the exact min/max union of its children.
    std::vector<float> nlo(3 * (size_t)ni), nhi(3 * (size_t)ni);
    std::vector<int> done(ni, 0);
    auto child_box = [&](int32_t c, float *blo_, float *bhi_) {
        if (c == ~0x7FFFFFFF) {
            for (int k = 0; k < 3; ++k) {
                blo_[k] = INFINITY;
                bhi_[k] = -INFINITY;
            }
        } else if (c < 0) {
            for (int k = 0; k < 3; ++k) {
                blo_[k] = s.leaf_lo[3 * (size_t)(~c) + k];
                bhi_[k] = s.leaf_hi[3 * (size_t)(~c) + k];
            }
        } else {
            for (int k = 0; k < 3; ++k) {
                blo_[k] = nlo[3 * (size_t)c + k];
                bhi_[k] = nhi[3 * (size_t)c + k];
            }
        }
    };
    std::vector<int> order;
    order.reserve(ni);
    // post-order via explicit stack
    {
        std::vector<std::pair<int, int>> st;
        st.push_back({0, 0});
        while (!st.empty()) {
            auto &top = st.back();
            int nd = top.first;
            if (top.second < 2) {
                int32_t c = s.nodes[nd].c[top.second++];
                if (c >= 0) st.push_back({c, 0});
            } else {
                order.push_back(nd);
                st.pop_back();
            }
        }
    }
    for (int nd : order) {
        float a0[3], b0[3], a1[3], b1[3];
        child_box(s.nodes[nd].c[0], a0, b0);
        child_box(s.nodes[nd].c[1], a1, b1);
        for (int k = 0; k < 3; ++k) {
            s.nodes[nd].b[k] = a0[k];
            s.nodes[nd].b[3 + k] = b0[k];
            s.nodes[nd].b[6 + k] = a1[k];
            s.nodes[nd].b[9 + k] = b1[k];
            nlo[3 * (size_t)nd + k] = std::fmin(a0[k], a1[k]);
            nhi[3 * (size_t)nd + k] = std::fmax(b0[k], b1[k]);
        }
    }
    (void)parent_internal;
    (void)parent_leaf;
    (void)done;
}

// Translucent covers (glass / plastic sheets; OptiX8DeviceCode.cu:793-911, materials from
// RadiationModel.cpp:2759-2807).  A primitive that is glass in EVERY band of a launch is a
// cover for that launch's rays of the source: it never stops them; each cover a ray crosses
// before its closest opaque hit (or the end of the periodic segment) attenuates the ray per
// band and receives the cover's own absorbed and reflected share.  The reference visits
// covers in OptiX any-hit order; here they are visited by increasing distance (ties: the
// smaller primitive index), at most kMaxCovers per segment.
constexpr int kMaxCovers = 16;
struct CoverQ {
    const uint32_t *bits = nullptr;  // [n] bit s: a cover for rays of source s (null: no covers)
    uint32_t cbit = 0;               // the ray's source bit
    int mode = 0;                    // 0: covers are transparent; 1: report only covers after (tlo, ilo)
    float tlo = -1.f;
    int32_t ilo = -1;
    int32_t self = -1;               // the ray's origin primitive, never its own cover
};

// Transmittance, reflectance and absorptance of one dielectric sheet of refractive index n
// and absorption product K*L at incidence cosine c: Fresnel reflection r at each face (s and
// p polarisation averaged), Bouguer attenuation ta along the refracted path and incoherent
// multiple reflections, T = ta (1-r)^2 / (1 - (r ta)^2), R = r (1 + ta T).  The physics of
// the reference's glass_tau_rho_alpha (OptiX8DeviceCode.cu:90-134, clamps kept), written in
// cosines.
inline void glass_trs(float c, float n, float KL, float *tau, float *rho, float *alpha) {
    c = std::fmin(1.f, std::fmax(1e-4f, c));
    const float st = std::sqrt(std::fmax(0.f, 1.f - c * c)) / n;
    const float ct = std::sqrt(std::fmax(0.f, 1.f - st * st));
    const float as = (c - n * ct) / (c + n * ct);
    const float ap = (n * c - ct) / (n * c + ct);
    const float ta = KL > 0.f ? std::exp(-KL / std::fmax(1e-4f, ct)) : 1.f;
    float T = 0.f, R = 0.f;
    for (int k = 0; k < 2; ++k) {
        const float r = k == 0 ? as * as : ap * ap;
        const float q = r * ta;
        const float den = std::fmax(1e-6f, 1.f - q * q);
        const float ti = ta * (1.f - r) * (1.f - r) / den;
        const float ri = r * (1.f + ta * ti);
        T += 0.5f * ti;
        R += 0.5f * ri;
    }
    T = std::fmax(0.f, std::fmin(1.f, T));
    R = std::fmax(0.f, std::fmin(1.f, R));
    *tau = T;
    *rho = R;
    *alpha = std::fmax(0.f, 1.f - T - R);
}

// Closest hit.  Ties in t go to the smaller original primitive index.
struct TraceStats {
    uint64_t nodes = 0, prims = 0;
};
inline bool better(float t, int32_t p, float bt, int32_t bp) {
    return t < bt || (t == bt && (uint32_t)p < (uint32_t)bp);
}

Hit trace_bvh(const Scene &s, const Ray &ray, bool anyhit, TraceStats *st, const CoverQ *cq = nullptr) {
    Hit h{ray.tmax, -1, 0};
    if (s.n == 0) return h;
    WT w = wt_setup(ray.d);
    V3 inv = v3(safe_inv(ray.d.x), safe_inv(ray.d.y), safe_inv(ray.d.z));
    V3 ooi = v3(ray.o.x * inv.x, ray.o.y * inv.y, ray.o.z * inv.z);
    int32_t stack[128];
    int sp = 0;
    int32_t cur = 0;
    float best = ray.tmax;
    for (;;) {
        const Node &nd = s.nodes[cur];
        if (st) st->nodes++;
        float tn0, tn1;
        bool h0 = slab_node(ooi, inv, v3(nd.b[0], nd.b[1], nd.b[2]), v3(nd.b[3], nd.b[4], nd.b[5]),
                            ray.tmin, best, &tn0);
        bool h1 = slab_node(ooi, inv, v3(nd.b[6], nd.b[7], nd.b[8]), v3(nd.b[9], nd.b[10], nd.b[11]),
                            ray.tmin, best, &tn1);
        int32_t c0 = nd.c[0], c1 = nd.c[1];
        // leaves are tested immediately, internal children are traversed near-first
        int32_t next[2];
        int nn = 0;
        for (int k = 0; k < 2; ++k) {
            bool hk = k == 0 ? h0 : h1;
            int32_t ck = k == 0 ? c0 : c1;
            if (!hk) continue;
            if (ck < 0) {
                if (ck == ~0x7FFFFFFF) continue;
                uint32_t slot = (uint32_t)(~ck);
                int32_t p = (int32_t)s.perm[slot];
                if (st) st->prims++;
                float t;
                int face;
                if (prim_hit(w, ray, inv, s.rec[p], (uint32_t)p, best, &t, &face, s.mk())) {
                    if (cq && cq->bits) {
                        const bool cov = (cq->bits[p] & cq->cbit) != 0;
                        if (cq->mode == 0 ? cov
                                          : (!cov || p == cq->self || !(t > cq->tlo || (t == cq->tlo && p > cq->ilo))))
                            continue;
                    }
                    if (h.prim < 0 || better(t, p, h.t, h.prim)) {
                        h.t = t;
                        h.prim = p;
                        h.face = face;
                        best = t;
                    }
                    if (anyhit) return h;
                }
            } else {
                next[nn++] = ck;
            }
        }
        if (nn == 2) {
            bool swap01 = tn1 < tn0;
            int32_t nearc = swap01 ? next[1] : next[0];
            int32_t farc = swap01 ? next[0] : next[1];
            stack[sp++] = farc;
            cur = nearc;
        } else if (nn == 1) {
            cur = next[0];
        } else {
            if (sp == 0) break;
            cur = stack[--sp];
        }
    }
    return h;
}

Hit trace_brute(const Scene &s, const Ray &ray, bool reference_formula) {
    Hit h{ray.tmax, -1, 0};
    WT w = wt_setup(ray.d);
    V3 inv = v3(safe_inv(ray.d.x), safe_inv(ray.d.y), safe_inv(ray.d.z));
    for (int p = 0; p < s.n; ++p) {
        float t;
        int face;
        bool ok = reference_formula
                      ? prim_hit_reference(ray, &s.T[16 * (size_t)p], (int)s.type[p], ray.tmax, &t, &face)
                      : prim_hit(w, ray, inv, s.rec[p], (uint32_t)p, ray.tmax, &t, &face, s.mk());
        if (ok && (h.prim < 0 || better(t, p, h.t, h.prim))) {
            h.t = t;
            h.prim = p;
            h.face = face;
        }
    }
    return h;
}

// Periodic walls: closest of the bbox faces (tested separately from the BVH).
inline bool bbox_closest(const Scene &s, const Ray &ray, float tmax, float *t_out, int *which) {
    if (s.nbbox == 0) return false;
    WT w = wt_setup(ray.d);
    bool any = false;
    float best = tmax;
    for (int b = 0; b < s.nbbox; ++b) {
        float t;
        int face;
        if (poly_hit(w, ray, s.bbox[b].p, 4, best, &t, &face)) {
            if (!any || t < best) {
                best = t;
                *which = b;
                any = true;
            }
        }
    }
    *t_out = best;
    return any;
}

// Full trace with periodic wrapping (<= 10 wraps, OptiX8DeviceCode.cu:1440-1459, 763-789).
Hit trace_full(const Scene &s, Ray ray, bool anyhit, TraceStats *st, V3 *o_last = nullptr) {
    const uint32_t c2 = ray.key.c2;
    for (int wrap = 0; wrap < 10; ++wrap) {
        ray.key.c2 = c2 | ((uint32_t)wrap << 16);
        if (o_last) *o_last = ray.o;
        Hit h = trace_bvh(s, ray, anyhit && s.nbbox == 0, st);
        if (s.nbbox == 0) return h;
        float tb;
        int which = -1;
        float lim = (h.prim >= 0) ? h.t : ray.tmax;
        if (!bbox_closest(s, ray, lim, &tb, &which) || (h.prim >= 0 && !(tb < h.t))) return h;
        // wrap to the opposite wall
        V3 hp = vadd(ray.o, vscale(ray.d, tb));
        bool xwall = (s.periodic[0] == 1.f) && which < 2;
        if (xwall) {
            float width = s.bbox[1].p[0].x - s.bbox[0].p[0].x;
            hp.x = hp.x + ((which == 0) ? width : -width);
        } else {
            int ybase = (s.periodic[0] == 1.f) ? 2 : 0;
            float width = s.bbox[ybase + 1].p[0].y - s.bbox[ybase].p[0].y;
            hp.y = hp.y + ((which == ybase) ? width : -width);
        }
        ray.o = hp;
    }
    // The tenth trace ended on a wall again: the reference's loop stops and neither a miss
    // nor a closest-hit program deposits energy for this ray (OptiX8DeviceCode.cu:1616-1653).
    return Hit{ray.tmax, -2, 0};
}

// trace_full for a launch with covers: closest opaque hit (covers transparent), then the
// covers of each periodic segment in order, reported to on_cover(prim, face).
template <class F>
Hit trace_covers(const Scene &s, Ray ray, const uint32_t *bits, uint32_t cbit, int32_t self, bool collect,
                 TraceStats *st, F &&on_cover) {
    const uint32_t c2 = ray.key.c2;
    CoverQ q0;
    q0.bits = bits;
    q0.cbit = cbit;
    for (int wrap = 0; wrap < 10; ++wrap) {
        ray.key.c2 = c2 | ((uint32_t)wrap << 16);
        Hit h = trace_bvh(s, ray, false, st, &q0);
        const float lim = (h.prim >= 0) ? h.t : ray.tmax;
        float tb = lim;
        int which = -1;
        const bool wall = s.nbbox > 0 && bbox_closest(s, ray, lim, &tb, &which) && (h.prim < 0 || tb < h.t);
        if (collect) {
            Ray seg = ray;
            seg.tmax = wall ? tb : lim;
            CoverQ q1 = q0;
            q1.mode = 1;
            q1.self = self;
            for (int c = 0; c < kMaxCovers; ++c) {
                Hit g = trace_bvh(s, seg, false, nullptr, &q1);
                if (g.prim < 0) break;
                on_cover(g.prim, g.face);
                q1.tlo = g.t;
                q1.ilo = g.prim;
            }
        }
        if (!wall) return h;
        V3 hp = vadd(ray.o, vscale(ray.d, tb));
        bool xwall = (s.periodic[0] == 1.f) && which < 2;
        if (xwall) {
            float width = s.bbox[1].p[0].x - s.bbox[0].p[0].x;
            hp.x = hp.x + ((which == 0) ? width : -width);
        } else {
            int ybase = (s.periodic[0] == 1.f) ? 2 : 0;
            float width = s.bbox[ybase + 1].p[0].y - s.bbox[ybase].p[0].y;
            hp.y = hp.y + ((which == ybase) ? width : -width);
        }
        ray.o = hp;
    }
    return Hit{ray.tmax, -2, 0};
}

// ---------------------------------------------------------------- sources ---
struct Source {
    int type;        // 0 collimated, 1 sphere, 2 sun sphere, 3 rectangle, 4 disk
    V3 pos;          // direction (collimated) or centre
    float w0, w1;    // width / diameter
    float R[9];      // rotation matrix (row-major) for rect / disk sources
};

// Sample origin on primitive p from uniform numbers u, v (and w, voxels only).
// Disks: concentric map onto the unit disk (OptiX 6 rayGeneration.cu:346-389 uses the
// same map); voxels: uniform in the box (rayGeneration.cu:391-396).
inline V3 sample_point(const RGen &g, int type, float u, float v, float w) {
    if (type == PT_TRI) {
        float a = u < v ? u : v, b = u < v ? v : u;  // sorted (OptiX8DeviceCode.cu:1288-1289)
        return v3((g.P.x + a * g.A.x) + b * g.B.x, (g.P.y + a * g.A.y) + b * g.B.y,
                  (g.P.z + a * g.A.z) + b * g.B.z);
    }
    if (type == PT_DISK) {
        float x, y;
        concentric(u, v, &x, &y);
        return v3((g.P.x + x * g.A.x) + y * g.B.x, (g.P.y + x * g.A.y) + y * g.B.y,
                  (g.P.z + x * g.A.z) + y * g.B.z);
    }
    if (type == PT_VOXEL)
        return v3(((g.P.x + u * g.A.x) + v * g.B.x) + w * g.N.x, ((g.P.y + u * g.A.y) + v * g.B.y) + w * g.N.y,
                  ((g.P.z + u * g.A.z) + v * g.B.z) + w * g.N.z);
    return v3((g.P.x + u * g.A.x) + v * g.B.x, (g.P.y + u * g.A.y) + v * g.B.y,
              (g.P.z + u * g.A.z) + v * g.B.z);
}

// Isotropic directions of a voxel's leaves: stratified uniform on the upper hemisphere
// (cos theta = 1 - Rt, OptiX 6 rayGeneration.cu:401-415); the bottom-face ray of the same
// sample takes the opposite direction, so each pair samples the sphere antithetically.
inline V3 voxel_dir(int ti, int pi, int dimx, int dimy, float j0, float j1) {
    float Rt = ((float)ti + j0) / (float)dimx;
    float Rp = ((float)pi + j1) / (float)dimy;
    float ct = 1.0f - Rt;
    float st = std::sqrt(std::fmax(0.f, 1.0f - ct * ct));
    float cp, sp;
    sincos2pi(Rp, &cp, &sp);
    return v3(st * cp, st * sp, ct);
}

// Leaf-projection factor of a direct ray's strength: |n . d| on a surface, G on a voxel.
inline double proj(V3 nrm, V3 d, bool vox) { return vox ? (double)kVoxelG : (double)std::fabs(vdot(nrm, d)); }

// Direction (and tmax, FP64 strength) of a direct ray towards source `src`
// (OptiX8DeviceCode.cu:1329-1415).  Returns false if the source emits away.
inline bool direct_dir(const Source &src, V3 org, V3 nrm, bool vox, uint32_t rx, uint32_t ry, double inv_nr,
                       V3 *dir, float *tmax, double *strength) {
    if (src.type == 0) {
        V3 d = vnormalize(src.pos);
        *dir = d;
        *tmax = 1e38f;
        *strength = inv_nr * proj(nrm, d, vox);
        return true;
    }
    if (src.type == 1 || src.type == 2) {
        float ct = 1.0f - 2.0f * u01(rx);
        float st = std::sqrt(std::fmax(0.f, 1.0f - ct * ct));
        float cp, sp;
        sincos2pi(u01(ry), &cp, &sp);
        float r = 0.5f * src.w0;
        V3 pt = v3(r * st * cp, r * st * sp, r * ct);
        V3 d = vsub(vadd(pt, src.pos), org);
        float dist = std::sqrt(vdot(d, d));
        d = vnormalize(d);
        double acc = 0.0;
        const int N = 10;
        for (int j = 0; j < N; ++j) {
            float cpj, spj;
            sincos2pi(((float)j + 0.5f) / (float)N, &cpj, &spj);
            for (int i = 0; i < N; ++i) {
                float cti = 1.0f - 2.0f * ((float)i + 0.5f) / (float)N;
                float sti = std::sqrt(std::fmax(0.f, 1.0f - cti * cti));
                V3 l = v3(sti * cpj, sti * spj, cti);
                if (vdot(l, d) < 0.f) {
                    acc += inv_nr * proj(nrm, d, vox) * (double)std::fabs(vdot(l, d)) /
                           ((double)dist * (double)dist) / (double)(N * N) * (double)src.w0 *
                           (double)src.w0;
                }
            }
        }
        *dir = d;
        *tmax = dist;
        *strength = acc;
        return true;
    }
    if (src.type == 3 || src.type == 4) {
        V3 pt;
        if (src.type == 3) {
            pt = v3(src.w0 * (-0.5f + u01(rx)), src.w1 * (-0.5f + u01(ry)), 0.f);
        } else {
            // concentric square-to-disk map (Shirley & Chiu 1997)
            float sx = -1.0f + 2.0f * u01(rx), sy = -1.0f + 2.0f * u01(ry);
            float r, ph;  // ph in units of pi/4
            if (sx > -sy) {
                if (sx > sy) { r = sx; ph = sy / sx; }
                else { r = sy; ph = 2.0f - sx / sy; }
            } else {
                if (sx < sy) { r = -sx; ph = 4.0f + sy / sx; }
                else { r = -sy; ph = (sy != 0.f) ? 6.0f - sx / sy : 0.f; }
            }
            float frac = ph * 0.125f;
            if (frac < 0.f) frac = frac + 1.0f;
            float c, s;
            sincos2pi(frac, &c, &s);
            pt = v3(src.w0 * r * c, src.w0 * r * s, 0.f);
        }
        const float *R = src.R;
        V3 q = v3((R[0] * pt.x + R[1] * pt.y) + R[2] * pt.z, (R[3] * pt.x + R[4] * pt.y) + R[5] * pt.z,
                  (R[6] * pt.x + R[7] * pt.y) + R[8] * pt.z);
        V3 ldir = v3(R[2], R[5], R[8]);
        V3 d = vsub(vadd(q, src.pos), org);
        if (vdot(d, ldir) > 0.f) return false;
        float dist = std::sqrt(vdot(d, d));
        d = vnormalize(d);
        double area = (src.type == 3) ? (double)src.w0 * (double)src.w1 / M_PI
                                      : (double)src.w0 * (double)src.w0;
        *strength = inv_nr * proj(nrm, d, vox) * (double)std::fabs(vdot(ldir, d)) /
                    ((double)dist * (double)dist) * area;
        *dir = d;
        *tmax = dist;
        return true;
    }
    return false;
}

// Diffuse (cosine-weighted, stratified) direction about normal n.
inline V3 diffuse_dir(V3 n, int ti, int pi, int dimx, int dimy, float j0, float j1) {
    float Rt = ((float)ti + j0) / (float)dimx;
    float Rp = ((float)pi + j1) / (float)dimy;
    float st = std::sqrt(Rt);
    float ct = std::sqrt(1.0f - Rt);
    float cp, sp;
    sincos2pi(Rp, &cp, &sp);
    float lx = st * cp, ly = st * sp;
    V3 t1, t2;
    onb(n, &t1, &t2);
    return v3((t1.x * lx + t2.x * ly) + n.x * ct, (t1.y * lx + t2.y * ly) + n.y * ct,
              (t1.z * lx + t2.z * ly) + n.z * ct);
}

// Origin of direct ray r of primitive p; u = philox(r, p, c2, 0; seed, pass) with c2 =
// source << 1.  Patches, disks and voxels are stratified in (u, v) over dimx x dimy cells
// (OptiX8DeviceCode.cu:1270-1290); a voxel's third coordinate comes from counter c2 | 1.
// Origins on masked primitives avoid transparent texels (OptiX8DeviceCode.cu:1252-1308):
// up to ten redraws, uniform over the primitive, from Philox counters
// (r, p, c2, 2^31 | attempt); the tenth redraw is kept unchecked, as in the reference.
inline void mask_origin(const Masks *mk, int type, uint32_t r, uint32_t p, uint32_t c2, uint32_t seed,
                        uint32_t pass, float *uu, float *vv) {
    if (!mk || mk->id[p] < 0 || !(type == PT_PATCH || type == PT_TILE || type == PT_TRI)) return;
    for (uint32_t a = 0; a < 10; ++a) {
        float fu, fv;
        if (type == PT_TRI) {
            float lo = *uu < *vv ? *uu : *vv, hi = *uu < *vv ? *vv : *uu;
            tri_uv(*mk, (int)p, hi - lo, lo, &fu, &fv);
        } else {
            patch_uv(*mk, (int)p, *uu - 0.5f, *vv - 0.5f, &fu, &fv);
        }
        if (mask_opaque(*mk, mk->id[p], fu, fv)) return;
        U4 q = draw(r, p, c2, 0x80000000u | (a + 1u), seed, pass);
        *uu = u01(q.v[0]);
        *vv = u01(q.v[1]);
    }
}

inline V3 direct_origin(const RGen &g, int type, uint32_t r, uint32_t p, uint32_t c2, int dimx, int dimy,
                        uint32_t seed, uint32_t pass, const U4 &u, const Masks *mk = nullptr) {
    float uu = u01(u.v[0]), vv = u01(u.v[1]), ww = 0.f;
    if (type != PT_TRI) {
        int xi = (int)(r % (uint32_t)dimx), yi = (int)(r / (uint32_t)dimx);
        uu = ((float)xi + uu) / (float)dimx;
        vv = ((float)yi + vv) / (float)dimy;
    }
    mask_origin(mk, type, r, p, c2, seed, pass, &uu, &vv);
    if (type == PT_VOXEL) ww = u01(draw(r, p, c2 | 1u, 0u, seed, pass).v[0]);
    return sample_point(g, type, uu, vv, ww);
}

// Origin and direction of diffuse ray r of primitive p leaving face `face` (1 top, 0
// bottom): cosine-weighted about the normal from counter (r, p, face, 0) on surfaces;
// on voxels both faces share the sample of counter (r, p, 1, 0) (third coordinate from
// (r, p, 2, 0)) and the bottom face flips the direction.
inline void diffuse_ray(const RGen &g, int type, uint32_t r, uint32_t p, int face, int dimx, int dimy,
                        uint32_t seed, uint32_t pass, V3 *org, V3 *dir, const Masks *mk = nullptr) {
    int ti = (int)(r % (uint32_t)dimx), pi = (int)(r / (uint32_t)dimx);
    V3 dd;
    if (type == PT_VOXEL) {
        U4 u = draw(r, p, 1u, 0u, seed, pass);
        U4 uw = draw(r, p, 2u, 0u, seed, pass);
        dd = voxel_dir(ti, pi, dimx, dimy, u01(u.v[0]), u01(u.v[1]));
        *org = sample_point(g, type, u01(u.v[2]), u01(u.v[3]), u01(uw.v[0]));
    } else {
        U4 u = draw(r, p, (uint32_t)face, 0u, seed, pass);
        dd = diffuse_dir(g.N, ti, pi, dimx, dimy, u01(u.v[0]), u01(u.v[1]));
        float uu = u01(u.v[2]), vv = u01(u.v[3]);
        mask_origin(mk, type, r, p, (uint32_t)face, seed, pass, &uu, &vv);
        *org = sample_point(g, type, uu, vv, 0.f);
    }
    *dir = (face == 0) ? v3(-dd.x, -dd.y, -dd.z) : dd;
}

// Material of primitive p as the deposits use it: a voxel's leaves scatter rho + tau,
// half of it routed to each face (both faces emit into the same isotropic field).
inline void eff_material(int type, float *rho, float *tau) {
    if (type == PT_VOXEL) {
        float h = 0.5f * (*rho + *tau);
        *rho = h;
        *tau = h;
    }
}

// Sky angular distribution (OptiX8DeviceCode.cu:148-164).
inline double sky_fd(V3 dir, V3 peak, float K, float knorm, const float *prague) {
    if (K > 0.f) {
        double c = std::max(-1.0, std::min(1.0, (double)vdot(peak, dir)));
        double psi = std::max(std::acos(c), M_PI / 180.0);
        return std::pow(psi, -(double)K) * (double)knorm;
    }
    if (prague[3] > 0.f) {
        double c = std::max(-1.0, std::min(1.0, (double)vdot(dir, peak)));
        double gamma = std::acos(c) * 180.0 / M_PI;
        double cth = std::max((double)dir.z, 0.0);
        double pat = (1.0 + prague[0] * std::exp(-gamma / prague[1])) * (1.0 + (prague[2] - 1.0) * (1.0 - cth));
        return pat * prague[3] * M_PI;
    }
    return 1.0;
}

// ---------------------------------------------------------------- cameras ---
// Camera and pixel-label rays (OptiX8DeviceCode.cu:1665-1812 generation, :673-741 miss,
// :1007-1170 closest hit, :743-748 and :1176-1199 pixel labels).  A camera ray of pixel
// (ii, jj), sample s, draws its sub-pixel offset and lens point from Philox counter
// (pixel, s, kCamCounter, 0) keyed by (seed, camera id), so images do not depend on tiling.
constexpr uint32_t kCamCounter = 0xCA3E0001u;
constexpr float kPiF = 3.14159265358979323846f;

struct Cam {
    V3 pos;
    float M[9];  // camera-to-world rotation, row-major; column 0 is the view axis
    float focal, lens, inv_aspect, L;
    int W, H, aa;
    uint32_t seed, id;
};

// Rotation of camera space (x = view axis) to the world for a view direction of the given
// zenith and azimuth: about y by zenith - pi/2, then about z by pi/2 - azimuth (the
// reference's d_rotatePoint), evaluated in FP64 and rounded to FP32.
inline void camera_rotation(float zenith, float azimuth, float M[9]) {
    const double th = -0.5 * M_PI + (double)zenith, ph = 0.5 * M_PI - (double)azimuth;
    const double st = std::sin(th), ct = std::cos(th), sp = std::sin(ph), cp = std::cos(ph);
    const double m[9] = {cp * ct, -sp, cp * st, sp * ct, cp, sp * st, -st, 0.0, ct};
    for (int i = 0; i < 9; ++i) M[i] = (float)m[i];
}

inline V3 mrot(const float M[9], V3 v) {
    return v3((M[0] * v.x + M[1] * v.y) + M[2] * v.z, (M[3] * v.x + M[4] * v.y) + M[5] * v.z,
              (M[6] * v.x + M[7] * v.y) + M[8] * v.z);
}

// Ray of pixel (ii, jj), sample s; centre: the pixel centre through the lens centre (labels).
inline void camera_ray(const Cam &c, uint32_t ii, uint32_t jj, uint32_t smp, bool centre, V3 *o, V3 *d) {
    float rx = 0.5f, ry = 0.5f, lx = 0.f, ly = 0.f;
    if (!centre) {
        U4 u = draw(jj * (uint32_t)c.W + ii, smp, kCamCounter, 0u, c.seed, c.id);
        rx = u01(u.v[0]);
        ry = u01(u.v[1]);
        if (c.lens > 0.f) concentric(u01(u.v[2]), u01(u.v[3]), &lx, &ly);
    }
    const float spy = -0.5f + ((float)ii + rx) / (float)c.W;
    const float spz = (0.5f - ((float)jj + ry) / (float)c.H) * c.inv_aspect;
    const V3 p = v3(c.focal, spy / c.L * c.focal, spz / c.L * c.focal);
    const V3 org = v3(0.f, 0.5f * lx * c.lens, 0.5f * ly * c.lens);
    *o = vadd(mrot(c.M, org), c.pos);
    *d = vnormalize(mrot(c.M, vsub(p, org)));
}

// Radiance of a sphere, rectangle or disk source seen along (o, d) before distance tlim
// (front faces only for rectangles and disks; OptiX8DeviceCode.cu:249-309, 1049-1126).
inline float source_radiance(const Source &sr, float flux, V3 o, V3 d, float tlim) {
    if (sr.type == 1) {
        const float r = 0.5f * sr.w0;
        const V3 oc = vsub(o, sr.pos);
        const float b = vdot(oc, d), cc = vdot(oc, oc) - r * r, disc = b * b - cc;
        if (disc < 0.f) return 0.f;
        const float t = -b - std::sqrt(disc);
        if (!(t > 0.f && t < tlim)) return 0.f;
        return flux / (4.f * kPiF * r * r) / kPiF;
    }
    if (sr.type == 3 || sr.type == 4) {
        const V3 n = v3(sr.R[2], sr.R[5], sr.R[8]);
        const float den = vdot(d, n);
        if (!(den < -1e-6f)) return 0.f;
        const float t = vdot(vsub(sr.pos, o), n) / den;
        if (!(t > 0.f && t < tlim)) return 0.f;
        const V3 hp = vsub(vadd(o, vscale(d, t)), sr.pos);
        float area;
        if (sr.type == 3) {
            const float lx = (sr.R[0] * hp.x + sr.R[3] * hp.y) + sr.R[6] * hp.z;
            const float ly = (sr.R[1] * hp.x + sr.R[4] * hp.y) + sr.R[7] * hp.z;
            if (std::fabs(lx) > 0.5f * sr.w0 || std::fabs(ly) > 0.5f * sr.w1) return 0.f;
            area = sr.w0 * sr.w1;
        } else {
            if (vdot(hp, hp) > sr.w0 * sr.w0) return 0.f;
            area = kPiF * sr.w0 * sr.w0;
        }
        return flux / area * (-den) / kPiF;
    }
    return 0.f;
}

// Camera view of the sky (RayTracingBackend::updateSkyModel): per launched band the sky
// radiance and Prague parameters, the solar disk, and the isotropic sky flux of emission bands.
struct CamSky {
    const float *sky_radiance = nullptr, *disk_radiance = nullptr, *diffuse_flux = nullptr, *prague = nullptr;
    const uint32_t *emission = nullptr;
    V3 sun = {0.f, 0.f, 1.f};
    float disk_cos = 0.f;
};

// Render one camera into pixels [W*H*Bl] (accumulated, FP64) and labels / depths [W*H].
void render_camera(const Scene &s, const Cam &c, int Bl, const std::vector<Source> &src, const float *src_flux,
                   const float *rtop, const float *rbot, const CamSky &sky, double *pix, uint32_t *labels,
                   float *depths) {
    const int S = (int)src.size();
    const float strength = 1.0f / (float)c.aa;
    const int np = c.W * c.H;
#pragma omp parallel for schedule(dynamic, 16)
    for (int q = 0; q < np; ++q) {
        const uint32_t ii = (uint32_t)(q % c.W), jj = (uint32_t)(q / c.W);
        for (int smp = 0; smp < c.aa; ++smp) {
            V3 o, d, ol;
            camera_ray(c, ii, jj, (uint32_t)smp, false, &o, &d);
            Hit h = trace_full(s, Ray{o, d, 1e-5f, 1e30f, VoxKey{(uint32_t)q, (uint32_t)smp, 0x40000000u, c.seed, c.id}},
                               false, nullptr, &ol);
            if (h.prim == -2) continue;
            for (int b = 0; b < Bl; ++b) {
                if (h.prim >= 0) {
                    const size_t ih = (size_t)h.prim * Bl + b;
                    float val = strength * (h.face ? rtop[ih] : rbot[ih]);
                    for (int k = 0; k < S; ++k) {
                        const float fl = src_flux[k * Bl + b];
                        if (!(fl > 0.f)) continue;
                        const float r = source_radiance(src[k], fl, ol, d, h.t);
                        if (r > 0.f) val += r * strength;
                    }
                    pix[(size_t)q * Bl + b] += (double)(val / kPiF);
                } else {
                    float rad = 0.f;
                    for (int k = 0; k < S; ++k) {
                        const float fl = src_flux[k * Bl + b];
                        if (!(fl > 0.f)) continue;
                        if (src[k].type == 0 || src[k].type == 2) {
                            if (sky.disk_radiance && sky.disk_radiance[b] > 0.f && vdot(d, sky.sun) >= sky.disk_cos)
                                rad += sky.disk_radiance[b];
                        } else {
                            rad += source_radiance(src[k], fl, ol, d, INFINITY);
                        }
                    }
                    if (rad <= 0.f && sky.sky_radiance && sky.sky_radiance[b] > 0.f) {
                        const float zero4[4] = {0.f, 0.f, 0.f, 0.f};
                        rad = sky.sky_radiance[b] * (float)sky_fd(d, sky.sun, 0.f, 1.f, sky.prague ? sky.prague + 4 * b : zero4);
                    }
                    if (sky.emission && sky.emission[b] && sky.diffuse_flux && sky.diffuse_flux[b] > 0.f)
                        rad += sky.diffuse_flux[b] / kPiF;
                    if (rad > 0.f) pix[(size_t)q * Bl + b] += (double)(rad * strength);
                }
            }
        }
        // pixel label and depth: the pixel centre through the lens centre
        V3 o, d, ol;
        camera_ray(c, ii, jj, 0u, true, &o, &d);
        Hit h = trace_full(s, Ray{o, d, 1e-5f, 1e30f, VoxKey{(uint32_t)q, 0xFFFFFFFFu, 0x40000000u, c.seed, c.id}},
                           false, nullptr, &ol);
        if (h.prim >= 0) {
            labels[q] = (uint32_t)h.prim + 1u;
            depths[q] = std::fabs(vdot(v3(c.M[0], c.M[3], c.M[6]), d)) * h.t;
        } else if (h.prim == -1) {
            labels[q] = 0u;
            depths[q] = -1.f;
        }
    }
}

}  // namespace

// ==================================================================== C API ===
extern "C" {

typedef struct {
    int32_t n;                // primitives
    const float *T;           // n*16 row-major transforms
    const uint32_t *type;     // n (0 patch, 1 triangle, 2 disk, 3 tile, 4 voxel)
    const int8_t *twosided;   // n (0 one-sided, 1 two-sided, 2 transparent, 3 skip)
    int32_t nbbox;            // periodic walls (0, 2 or 4)
    const float *bbox_verts;  // nbbox*4*3 world-space corners
    float periodic_x, periodic_y;
    const float *voxel_lad;   // n leaf area density (m^2/m^3), read for voxels; may be null without voxels
    const int32_t *mask_id;   // n texture mask of each primitive (-1 none), or null: no masks
    const int32_t *uv_id;     // n >= 0: uv holds the primitive's texture coordinates
    const float *uv;          // n*8 corner (u,v) pairs, or null
    int32_t nmasks;
    const int32_t *mask_size; // nmasks*2 width, height
    const uint8_t *mask_data; // all masks, row-major, nonzero = opaque
} orc_geometry;

typedef struct {
    int32_t nbands_global;
    const uint8_t *band_launch;   // [nbands_global]
    int32_t nsources;
    const int32_t *source_type;   // [S]
    const float *source_pos;      // [S*3]
    const float *source_width;    // [S*2]
    const float *source_rot;      // [S*9] rotation matrices (row-major) for rect/disk
    const float *source_flux;     // [S*Bl]
    const float *rho;             // [S*n*Bg]
    const float *tau;             // [S*n*Bg]
    const float *diffuse_flux;    // [Bl]
    const float *diffuse_ext;     // [Bl] power-law K (0 = off)
    const float *diffuse_norm;    // [Bl]
    const float *diffuse_peak;    // [Bl*3]
    const float *prague;          // [Bl*4]
    const int32_t *direct_rays;   // [Bl]
    const int32_t *diffuse_rays;  // [Bl]
    const int32_t *depth;         // [Bl]
    const uint8_t *emission;      // [Bl]
    const float *eps;             // [n*Bl] emissivity (after RadiationModel's rules)
    const float *temperature;     // [n] K
    uint32_t seed;
    int32_t threads;              // OpenMP threads (<=0: all)
    int32_t prim_limit;           // >0: launch rays only from the first prim_limit primitives (timing samples)
    double scatter_tol;           // >0: a band stops scattering once its residual falls to this value
    int32_t glass_nsrc;           // sources of the glass arrays (0: no translucent covers)
    const int8_t *is_glass;       // [glass_nsrc*n*Bg]
    const float *glass_n;         // [glass_nsrc*n*Bg] refractive index
    const float *glass_kl;        // [glass_nsrc*n*Bg] absorption product K*L
    int32_t ncameras;             // cameras rendered after the solve (needs scattering enabled)
    const struct orc_camera *cameras;
    const float *cam_sky_radiance;  // [Bl] camera sky model, each may be null
    const float *cam_disk_radiance; // [Bl]
    const float *cam_diffuse_flux;  // [Bl]
    const float *cam_prague;        // [Bl*4]
    const uint32_t *cam_emission;   // [Bl]
    float cam_sun[3];
    float cam_disk_cos;
} orc_solve;

typedef struct orc_camera {
    float position[3];
    float direction[2];           // zenith, azimuth of the view axis (radians)
    float focal_length, lens_diameter, fov_aspect, viewplane_length;
    int32_t width, height, antialiasing;
    uint32_t seed, camera_id;
    float *pixels;                // out [W*H*Bl] radiance
    uint32_t *labels;             // out [W*H] primitive index + 1 (0: sky)
    float *depths;                // out [W*H] depth along the view axis (-1: sky)
} orc_camera;

void *orc_scene_create(const orc_geometry *g) {
    Scene *s = new Scene();
    s->n = g->n;
    s->T.assign(g->T, g->T + 16 * (size_t)g->n);
    s->type.assign(g->type, g->type + g->n);
    s->twosided.assign(g->twosided, g->twosided + g->n);
    s->rec.resize(g->n);
    s->rgen.resize(g->n);
    s->area.resize(g->n);
    for (int i = 0; i < g->n; ++i) {
        float lad = 0.f;
        if (s->type[i] == PT_VOXEL) {
            if (!g->voxel_lad) {
                delete s;
                return nullptr;
            }
            lad = g->voxel_lad[i];
            s->twosided[i] = 1;  // a voxel launches both ray directions of each sample
        }
        s->rec[i] = make_rec(&s->T[16 * (size_t)i], (int)s->type[i], lad);
        s->rgen[i] = make_rgen(&s->T[16 * (size_t)i], (int)s->type[i]);
        s->area[i] = prim_area(&s->T[16 * (size_t)i], (int)s->type[i], lad);
    }
    if (g->mask_id && g->nmasks > 0) {
        Masks &m = s->masks;
        m.id.assign(g->mask_id, g->mask_id + g->n);
        m.uv_id.assign(g->n, -1);
        if (g->uv_id && g->uv) {
            m.uv_id.assign(g->uv_id, g->uv_id + g->n);
            m.uv.assign(g->uv, g->uv + 8 * (size_t)g->n);
        }
        m.size.assign(g->mask_size, g->mask_size + 2 * (size_t)g->nmasks);
        uint32_t off = 0;
        for (int k = 0; k < g->nmasks; ++k) {
            m.offset.push_back(off);
            off += (uint32_t)(m.size[2 * k] * m.size[2 * k + 1]);
        }
        m.data.assign(g->mask_data, g->mask_data + off);
        m.T = s->T.data();
    }
    s->nbbox = g->nbbox;
    s->periodic[0] = g->periodic_x;
    s->periodic[1] = g->periodic_y;
    for (int b = 0; b < g->nbbox; ++b) {
        Rec r{};
        r.type = PT_BBOX;
        for (int v = 0; v < 4; ++v)
            r.p[v] = v3(g->bbox_verts[12 * b + 3 * v], g->bbox_verts[12 * b + 3 * v + 1],
                        g->bbox_verts[12 * b + 3 * v + 2]);
        s->bbox.push_back(r);
    }
    if (s->n > 0) build_bvh(*s);
    return s;
}

void orc_scene_destroy(void *h) { delete (Scene *)h; }

// Philox4x32-10 block (for known-answer tests).
// Random-number stream of the ray generators: 0 Philox (default), 1 the reference's TEA + LCG.
int orc_set_rng(int mode) {
    if (mode != 0 && mode != 1) return -1;
    g_rng_mode = mode;
    return 0;
}

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    U4 u = philox(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = u.v[i];
}

// sincos2pi for a batch (tests of the polynomial against libm).
void orc_sincos2pi(int64_t n, const float *u, float *c, float *s) {
    for (int64_t i = 0; i < n; ++i) sincos2pi(u[i], &c[i], &s[i]);
}

// ln_unit for a batch (accuracy tests against libm).
// Surface energy balance (plugins/energybalance/src/EnergyBalanceModel.cu:34-125, outputs
// :466-505): per primitive, the secant root from (Tin, 400 K) of R - Nsides eps sigma T^4 - QH -
// QL - Qother - storage, relative step 1e-4, at most 100 steps, in FP32 as the reference computes
// it.  in: [11][n] Ta, ea, P, gH, gS, eps, Qother, C, hs, sidedness, R; returns the number of
// primitives that did not converge.  out5 (may be null): [n][5] sensible, latent, storage, net
// radiation, vapour pressure deficit / P.
int orc_energy_balance(int32_t n, const float *in, const uint8_t *nsides, const float *Tin, float dt, float Tdef,
                       float *Tout, float *out5) {
    const float cp = 29.25f, lam = 44000.f, sig = 5.67e-8f;
    const size_t N = (size_t)n;
    int bad = 0;
    for (int32_t p = 0; p < n; ++p) {
        const float Ta = in[p], ea = in[N + p], P = in[2 * N + p], gH = in[3 * N + p], gS = in[4 * N + p],
                    eps = in[5 * N + p], Qo = in[6 * N + p], C = in[7 * N + p], hs = in[8 * N + p],
                    sd = in[9 * N + p], R = in[10 * N + p];
        const float ns = (float)nsides[p];
        const float gM = (gH == 0.f || gS == 0.f)
                             ? 0.f
                             : 1.08f * gH * gS * (sd / (1.08f * gH + gS * sd) + (1.f - sd) / (1.08f * gH + gS * (1.f - sd)));
        const float Tprev = Tin[p];
        auto res = [&](float T) {
            const float Rout = ns * eps * sig * T * T * T * T;
            const float QH = cp * gH * (T - Ta);
            const float es = 611.0f * std::exp(17.502f * (T - 273.f) / (T - 273.f + 240.97f));
            const float QL = gM * lam * (es - ea * hs) / P;
            const float st = dt > 0.f ? C * (T - Tprev) / dt : 0.f;
            return R - Rout - QH - QL - Qo - st;
        };
        float T0 = Tprev, T1 = 400.f;
        if (T1 == T0) T1 = T0 + 100.f;
        float T = T0, r0 = res(T0), r1 = res(T1), err = 100.f;
        for (int it = 0; it < 100 && err > 1e-4f; ++it) {
            if (r0 == r1) {
                err = 0.f;
                break;
            }
            T = std::fabs((T1 * r0 - T0 * r1) / (r0 - r1));
            const float r = res(T);
            err = std::fabs(T - T0) / std::fabs(T0);
            r1 = r0;
            r0 = r;
            T1 = T0;
            T0 = T;
        }
        if (!std::isfinite(T)) T = Tdef;
        if (err > 1e-4f) ++bad;
        Tout[p] = T;
        if (out5) {
            const float es = 611.0f * std::exp(17.502f * (T - 273.15f) / (T - 273.15f + 240.97f));
            float *o = out5 + 5 * (size_t)p;
            o[0] = cp * gH * (T - Ta);
            o[1] = lam * gM * (es - ea) / P;
            o[2] = dt > 0.f ? C * (T - Tprev) / dt : 0.f;
            o[3] = R - ns * eps * sig * T * T * T * T;
            o[4] = (es - ea) / P;
        }
    }
    return bad;
}

void orc_glass_trs(int64_t m, const float *c, float n, float kl, float *out) {
    for (int64_t i = 0; i < m; ++i) glass_trs(c[i], n, kl, &out[3 * i], &out[3 * i + 1], &out[3 * i + 2]);
}

void orc_ln_unit(int64_t n, const float *x, float *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = ln_unit(x[i]);
}

// Export the host-built BVH for bit-exact comparison with the device build.
// nodes: (n-1) * 16 words: 12 float box words then child0, child1, 0, 0.
int orc_scene_bvh(void *h, uint64_t *codes, uint32_t *perm, uint32_t *nodes) {
    Scene *s = (Scene *)h;
    if (s->n == 0) return 0;
    std::memcpy(codes, s->codes.data(), sizeof(uint64_t) * s->n);
    std::memcpy(perm, s->perm.data(), sizeof(uint32_t) * s->n);
    for (size_t i = 0; i < s->nodes.size(); ++i) {
        std::memcpy(&nodes[16 * i], s->nodes[i].b, 48);
        nodes[16 * i + 12] = (uint32_t)s->nodes[i].c[0];
        nodes[16 * i + 13] = (uint32_t)s->nodes[i].c[1];
        nodes[16 * i + 14] = 0;
        nodes[16 * i + 15] = 0;
    }
    return (int)s->nodes.size();
}

// Closest hit for explicit rays.  mode 0: BVH + watertight; 1: brute force + watertight;
// 2: brute force + reference formulas; 3: BVH any-hit.  counters (may be null):
// [0] node visits, [1] primitive tests (BVH modes only).
int orc_trace(void *h, int64_t nrays, const float *o, const float *d, float tmin, float tmax, int mode,
              int32_t *hit, float *t, int32_t *face, uint64_t *counters, int threads) {
    Scene *s = (Scene *)h;
    uint64_t cn = 0, cp = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : cn, cp)
    for (int64_t i = 0; i < nrays; ++i) {
        // voxel draws of explicit ray i: counter (i, i >> 32, 2^31), key (0, ~0)
        Ray r{v3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), v3(d[3 * i], d[3 * i + 1], d[3 * i + 2]), tmin, tmax,
              VoxKey{(uint32_t)i, (uint32_t)((uint64_t)i >> 32), 0x80000000u, 0u, 0xFFFFFFFFu}};
        Hit hh;
        TraceStats st;
        if (mode == 0 || mode == 3) hh = trace_bvh(*s, r, mode == 3, &st);
        else hh = trace_brute(*s, r, mode == 2);
        hit[i] = hh.prim;
        if (t) t[i] = hh.t;
        if (face) face[i] = hh.face;
        cn += st.nodes;
        cp += st.prims;
    }
    if (counters) {
        counters[0] = cn;
        counters[1] = cp;
    }
    return 0;
}

// Generate the ray set of one pass, for hit-ID parity.
// kind 0: direct rays toward collimated direction dir3 (one per stratum, rpp rays per prim);
// kind 1: diffuse rays (top face, rpp rays per prim).  Outputs n*rpp rays (origin, dir).
int orc_gen_rays(void *h, int kind, uint32_t seed, uint32_t pass, int32_t rpp, int32_t face,
                 const float *dir3, float *o, float *d) {
    Scene *s = (Scene *)h;
    int dimx = (int)std::sqrt((float)rpp);
    if (dimx < 1) dimx = 1;
    int dimy = rpp / dimx;
    int nr = dimx * dimy;
    for (int p = 0; p < s->n; ++p) {
        const RGen &g = s->rgen[p];
        for (int r = 0; r < nr; ++r) {
            V3 org, dir;
            if (kind == 0) {
                U4 u = draw((uint32_t)r, (uint32_t)p, (uint32_t)face, 0u, seed, pass);
                org = direct_origin(g, (int)s->type[p], (uint32_t)r, (uint32_t)p, (uint32_t)face, dimx, dimy, seed,
                                    pass, u, s->mk());
                dir = vnormalize(v3(dir3[0], dir3[1], dir3[2]));
            } else {
                diffuse_ray(g, (int)s->type[p], (uint32_t)r, (uint32_t)p, face, dimx, dimy, seed, pass, &org, &dir,
                            s->mk());
            }
            size_t k = (size_t)p * nr + r;
            o[3 * k] = org.x;
            o[3 * k + 1] = org.y;
            o[3 * k + 2] = org.z;
            d[3 * k] = dir.x;
            d[3 * k + 1] = dir.y;
            d[3 * k + 2] = dir.z;
        }
    }
    return nr;
}

// --------------------------------------------------------------- runBand ---
// Restatement of RadiationModel::runBand (RadiationModel.cpp:3470-4663) driving the
// OptiX8 device-program semantics, with FP64 buffers.  flux_out: [n*Bl] =
// radiation_in + scatter_top + scatter_bottom (RadiationModel.cpp:4652).
// stats (may be null): [0] rays traced, [1] BVH node visits, [2] primitive tests, [3] hits,
// [4] scattering iterations run.
int orc_run_band(void *h, const orc_solve *q, double *flux_out, uint64_t *stats) {
    Scene *s = (Scene *)h;
    const int n = s->n;
    const int Bg = q->nbands_global;
    int Bl = 0;
    for (int b = 0; b < Bg; ++b) Bl += q->band_launch[b] ? 1 : 0;
    const int S = q->nsources;
#ifdef _OPENMP
    if (q->threads > 0) omp_set_num_threads(q->threads);
#endif
    std::vector<double> rin((size_t)n * Bl, 0.0), otop((size_t)n * Bl, 0.0), obot((size_t)n * Bl, 0.0),
        stop((size_t)n * Bl, 0.0), sbot((size_t)n * Bl, 0.0);
    std::vector<Source> src(S);
    for (int k = 0; k < S; ++k) {
        src[k].type = q->source_type[k];
        src[k].pos = v3(q->source_pos[3 * k], q->source_pos[3 * k + 1], q->source_pos[3 * k + 2]);
        src[k].w0 = q->source_width[2 * k];
        src[k].w1 = q->source_width[2 * k + 1];
        for (int i = 0; i < 9; ++i) src[k].R[i] = q->source_rot ? q->source_rot[9 * k + i] : (i % 4 == 0 ? 1.f : 0.f);
    }
    bool rundirect = false;
    for (int k = 0; k < S; ++k)
        for (int b = 0; b < Bl; ++b)
            if (q->source_flux[k * Bl + b] > 0.f) rundirect = true;
    bool scattering = false, diffuse = false, emission = false;
    int dirN = 0, difN = 0, depth = 0;
    for (int b = 0; b < Bl; ++b) {
        scattering = scattering || q->depth[b] > 0;
        diffuse = diffuse || q->diffuse_flux[b] > 0.f;
        emission = emission || q->emission[b];
        dirN = std::max(dirN, q->direct_rays[b]);
        difN = std::max(difN, q->diffuse_rays[b]);
        depth = std::max(depth, q->depth[b]);
    }
    uint64_t n_rays = 0, n_nodes = 0, n_prims = 0, n_hits = 0;
    int iters = 0;
    const int nl = (q->prim_limit > 0 && q->prim_limit < n) ? q->prim_limit : n;
    auto matidx = [&](int srcid, int p, int bg) { return ((size_t)srcid * n + p) * Bg + bg; };
    // Cover bits of one launch: bit k of primitive p when p is glass for source k in every
    // launched band (voxels never are); empty when no primitive is a cover.
    auto cover_bits = [&](const uint8_t *fl, int nsrc) {
        std::vector<uint32_t> bits;
        if (!q->is_glass || q->glass_nsrc <= 0) return bits;
        bits.assign(n, 0u);
        bool any = false;
        const int ns = std::min(std::min(nsrc, q->glass_nsrc), 32);
        for (int p = 0; p < n; ++p) {
            if (s->type[p] == PT_VOXEL) continue;
            for (int k = 0; k < ns; ++k) {
                bool launched = false, all = true;
                for (int bg = 0; bg < Bg && all; ++bg) {
                    if (!fl[bg]) continue;
                    launched = true;
                    all = q->is_glass[matidx(k, p, bg)] != 0;
                }
                if (launched && all) {
                    bits[p] |= 1u << k;
                    any = true;
                }
            }
        }
        if (!any) bits.clear();
        return bits;
    };
    // A cover's absorbed and reflected shares of `incoming` (OptiX8DeviceCode.cu:874-895).
    auto cover_deposit = [&](int c, int face, int b, double incoming, float alpha, float rho) {
        if (!(incoming > 0.0)) return;
        const size_t i = (size_t)c * Bl + b;
#pragma omp atomic
        rin[i] += incoming * (double)alpha;
        double *sc = face ? &stop[i] : &sbot[i];
#pragma omp atomic
        *sc += incoming * (double)rho;
    };

    // ---- direct pass (OptiX8Backend::launchDirectRays + __raygen__direct + __miss__direct)
    if (S > 0 && rundirect && dirN > 0) {
        int dimx = (int)std::sqrt((float)dirN);
        int dimy = dimx > 0 ? dirN / dimx : 1;
        double inv_nr = 1.0 / (double)(dimx * dimy);
        const std::vector<uint32_t> dbits = cover_bits(q->band_launch, S);
        const uint32_t *cb = dbits.empty() ? nullptr : dbits.data();
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : n_rays, n_nodes, n_prims, n_hits)
        for (int p = 0; p < nl; ++p) {
            const RGen &g = s->rgen[p];
            int ts = s->twosided[p];
            std::vector<double> d_in(Bl, 0.0), d_top(Bl, 0.0), d_bot(Bl, 0.0);
            std::vector<float> ctau(Bl, 1.f);
            const int type = (int)s->type[p];
            const bool vox = type == PT_VOXEL;
            for (int r = 0; r < dimx * dimy; ++r) {
                for (int k = 0; k < S; ++k) {
                    const uint32_t c2 = (uint32_t)(k << 1);
                    U4 u = draw((uint32_t)r, (uint32_t)p, c2, 0u, q->seed, 0u);
                    V3 org = direct_origin(g, type, (uint32_t)r, (uint32_t)p, c2, dimx, dimy, q->seed, 0u, u, s->mk());
                    V3 dir;
                    float tmax;
                    double strength;
                    if (!direct_dir(src[k], org, g.N, vox, u.v[2], u.v[3], inv_nr, &dir, &tmax, &strength)) continue;
                    bool face = vox || vdot(dir, g.N) > 0.f;
                    if (!face && ts == 0) continue;
                    if (ts == 3) continue;
                    TraceStats st;
                    const Ray ray{org, dir, 1e-4f, tmax, VoxKey{(uint32_t)r, (uint32_t)p, c2, q->seed, 0u}};
                    Hit hh;
                    if (!cb) {
                        hh = trace_full(*s, ray, true, &st);
                    } else {
                        std::fill(ctau.begin(), ctau.end(), 1.f);
                        hh = trace_covers(*s, ray, cb, 1u << k, p, true, &st, [&](int c, int cface) {
                            const float cs = std::fmin(1.f, std::fabs(vdot(dir, s->rgen[c].N)));
                            int b = -1;
                            for (int bg = 0; bg < Bg; ++bg) {
                                if (!q->band_launch[bg]) continue;
                                ++b;
                                float tau_c, rho_c, alpha_c;
                                glass_trs(cs, q->glass_n[matidx(k, c, bg)], q->glass_kl[matidx(k, c, bg)], &tau_c,
                                          &rho_c, &alpha_c);
                                cover_deposit(c, cface, b,
                                              strength * (double)q->source_flux[k * Bl + b] * (double)ctau[b],
                                              alpha_c, rho_c);
                                ctau[b] *= tau_c;
                            }
                        });
                    }
                    n_rays++;
                    n_nodes += st.nodes;
                    n_prims += st.prims;
                    if (hh.prim >= 0) n_hits++;
                    if (hh.prim != -1) continue;  // occluded, or dropped at the wrap limit
                    int b = -1;
                    for (int bg = 0; bg < Bg; ++bg) {
                        if (!q->band_launch[bg]) continue;
                        ++b;
                        float rho = q->rho[matidx(k, p, bg)], tau = q->tau[matidx(k, p, bg)];
                        eff_material(type, &rho, &tau);
                        double str = strength * (double)q->source_flux[k * Bl + b];
                        if (cb) str *= (double)ctau[b];
                        d_in[b] += str * (1.0 - rho - tau);
                        if (rho > 0.f || tau > 0.f) {
                            if (face) {
                                d_top[b] += str * rho;
                                d_bot[b] += str * tau;
                            } else {
                                d_bot[b] += str * rho;
                                d_top[b] += str * tau;
                            }
                        }
                    }
                }
            }
            for (int b = 0; b < Bl; ++b) {  // atomic: covers deposit on other primitives concurrently
#pragma omp atomic
                rin[(size_t)p * Bl + b] += d_in[b];
#pragma omp atomic
                stop[(size_t)p * Bl + b] += d_top[b];
#pragma omp atomic
                sbot[(size_t)p * Bl + b] += d_bot[b];
            }
        }
    }

    // ---- diffuse launch (OptiX8Backend::launchDiffuseRays + __raygen__diffuse +
    //      __closesthit__diffuse / __miss__diffuse); flags = launched-band mask
    auto diffuse_pass = [&](int face, uint32_t pass, const std::vector<uint8_t> &flags,
                            const std::vector<float> &dflux) {
        int rpp = (int)std::ceil(std::sqrt((double)difN));
        rpp = rpp * rpp;
        if (rpp == 0 || n == 0) return;
        int dimx = (int)std::sqrt((float)rpp);
        int dimy = dimx > 0 ? rpp / dimx : 1;
        double strength = 1.0 / (double)(dimx * dimy);
        const std::vector<uint32_t> fbits = cover_bits(flags.data(), 1);
        const uint32_t *cb = fbits.empty() ? nullptr : fbits.data();
        bool sky = false;
        for (int b = 0; b < Bl; ++b) sky = sky || dflux[b] > 0.f;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : n_rays, n_nodes, n_prims, n_hits)
        for (int p = 0; p < nl; ++p) {
            int ts = s->twosided[p];
            if (face == 0 && ts == 0) continue;
            if (face == 1 && ts == 3) continue;
            if (face == 0 && ts != 1) continue;
            const RGen &g = s->rgen[p];
            const int type = (int)s->type[p];
            // a voxel's two ray directions both deposit on its top face
            const int dface = (type == PT_VOXEL) ? 1 : face;
            std::vector<double> d_in(Bl, 0.0), d_top(Bl, 0.0), d_bot(Bl, 0.0);
            std::vector<float> ctau(Bl, 1.f);
            for (int r = 0; r < dimx * dimy; ++r) {
                V3 org, dir;
                diffuse_ray(g, type, (uint32_t)r, (uint32_t)p, face, dimx, dimy, q->seed, pass, &org, &dir, s->mk());
                TraceStats st;
                const Ray ray{org, dir, 1e-4f, 1e38f, VoxKey{(uint32_t)r, (uint32_t)p, (uint32_t)face, q->seed, pass}};
                Hit hh;
                if (!cb) {
                    hh = trace_full(*s, ray, false, &st);
                } else {
                    // covers deposit the isotropic sky flux of the launch (OptiX8DeviceCode.cu:871-880)
                    std::fill(ctau.begin(), ctau.end(), 1.f);
                    hh = trace_covers(*s, ray, cb, 1u, p, sky, &st, [&](int c, int cface) {
                        const float cs = std::fmin(1.f, std::fabs(vdot(dir, s->rgen[c].N)));
                        int b = -1;
                        for (int bg = 0; bg < Bg; ++bg) {
                            if (!flags[bg]) continue;
                            ++b;
                            float tau_c, rho_c, alpha_c;
                            glass_trs(cs, q->glass_n[matidx(0, c, bg)], q->glass_kl[matidx(0, c, bg)], &tau_c, &rho_c,
                                      &alpha_c);
                            cover_deposit(c, cface, b, strength * (double)dflux[b] * (double)ctau[b], alpha_c, rho_c);
                            ctau[b] *= tau_c;
                        }
                    });
                }
                n_rays++;
                n_nodes += st.nodes;
                n_prims += st.prims;
                if (hh.prim >= 0) n_hits++;
                if (hh.prim == -2) continue;  // dropped at the wrap limit: no deposit
                int b = -1;
                for (int bg = 0; bg < Bg; ++bg) {
                    if (!flags[bg]) continue;
                    ++b;
                    double val;
                    if (hh.prim >= 0) {
                        size_t ih = (size_t)hh.prim * Bl + b;
                        val = (hh.face ? otop[ih] : obot[ih]) * strength;
                        if (val == 0.0) continue;
                    } else {
                        if (!(dflux[b] > 0.f)) continue;
                        V3 pk = q->diffuse_peak ? v3(q->diffuse_peak[3 * b], q->diffuse_peak[3 * b + 1], q->diffuse_peak[3 * b + 2])
                                                : v3(0.f, 0.f, 1.f);
                        float K = q->diffuse_ext ? q->diffuse_ext[b] : 0.f;
                        float kn = q->diffuse_norm ? q->diffuse_norm[b] : 1.f;
                        float zero4[4] = {0, 0, 0, 0};
                        const float *pr = q->prague ? &q->prague[4 * b] : zero4;
                        val = sky_fd(dir, pk, K, kn, pr) * (double)dflux[b] * strength;
                        if (cb) val *= (double)ctau[b];
                    }
                    float rho = q->rho[matidx(0, p, bg)], tau = q->tau[matidx(0, p, bg)];
                    eff_material(type, &rho, &tau);
                    d_in[b] += val * (1.0 - rho - tau);
                    if (rho > 0.f || tau > 0.f) {
                        if (dface) {
                            d_top[b] += val * rho;
                            d_bot[b] += val * tau;
                        } else {
                            d_bot[b] += val * rho;
                            d_top[b] += val * tau;
                        }
                    }
                }
            }
            for (int b = 0; b < Bl; ++b) {  // atomic: covers deposit on other primitives concurrently
#pragma omp atomic
                rin[(size_t)p * Bl + b] += d_in[b];
#pragma omp atomic
                stop[(size_t)p * Bl + b] += d_top[b];
#pragma omp atomic
                sbot[(size_t)p * Bl + b] += d_bot[b];
            }
        }
    };

    std::vector<uint8_t> flags(q->band_launch, q->band_launch + Bg);
    std::vector<float> dflux(q->diffuse_flux, q->diffuse_flux + Bl);
    std::vector<double> ftop((size_t)n * Bl, 0.0), fbot((size_t)n * Bl, 0.0);
    // Camera view of the primitives: the scatter of every pass plus emission, accumulated
    // (RadiationModel.cpp:3992-4012, 4105-4131, 4211-4220, 4336-4345).
    const bool cams = q->ncameras > 0 && q->cameras;
    std::vector<double> ctop, cbot;
    if (cams) {
        ctop.assign((size_t)n * Bl, 0.0);
        cbot.assign((size_t)n * Bl, 0.0);
    }
    auto cam_add_scatter = [&]() {
        if (!cams) return;
        for (size_t i = 0; i < ctop.size(); ++i) {
            ctop[i] += stop[i];
            cbot[i] += sbot[i];
        }
    };
    if (scattering && rundirect) {
        cam_add_scatter();
        ftop = stop;
        fbot = sbot;
        for (int p = 0; p < n; ++p) {
            if (s->twosided[p] != 0) continue;
            for (int b = 0; b < Bl; ++b) {
                size_t i = (size_t)p * Bl + b;
                double tot = ftop[i] + fbot[i];
                ftop[i] = tot;
                fbot[i] = tot;
            }
        }
        otop = ftop;
        obot = fbot;
        std::fill(stop.begin(), stop.end(), 0.0);
        std::fill(sbot.begin(), sbot.end(), 0.0);
    }
    if (emission || diffuse) {
        if (emission) {
            const float sigma = 5.6703744e-8f;
            for (int b = 0; b < Bl; ++b) {
                if (!q->emission[b]) continue;
                for (int p = 0; p < n; ++p) {
                    float eps = q->eps[(size_t)p * Bl + b];
                    if (q->depth[b] == 0 && eps != 1.f) eps = 1.f;
                    double T = (double)q->temperature[p];
                    float out = (float)((double)(sigma * eps) * (T * T * T * T));
                    size_t i = (size_t)p * Bl + b;
                    ftop[i] += out;
                    if (s->twosided[p] != 0) fbot[i] += out;
                    if (cams) {
                        ctop[i] += out;
                        if (s->twosided[p] != 0) cbot[i] += out;
                    }
                }
            }
        }
        otop = ftop;
        obot = fbot;
        diffuse_pass(1, 1u, flags, dflux);
        diffuse_pass(0, 1u, flags, dflux);
        cam_add_scatter();
    }
    if (scattering && (emission || diffuse) && !rundirect) {
        otop = stop;
        obot = sbot;
        std::fill(stop.begin(), stop.end(), 0.0);
        std::fill(sbot.begin(), sbot.end(), 0.0);
    }
    if (scattering && (emission || diffuse || rundirect)) {
        std::fill(dflux.begin(), dflux.end(), 0.f);
        std::vector<uint8_t> sflags = flags;
        std::vector<uint8_t> conv(Bg, 0);
        for (int it = 0; it < depth; ++it) {
            int b = -1;
            for (int bg = 0; bg < Bg; ++bg) {
                if (!sflags[bg]) continue;
                ++b;
                if (it + 1 > q->depth[b] || conv[bg]) sflags[bg] = 0;
            }
            if (it > 0 || (emission && rundirect)) {
                otop = stop;
                obot = sbot;
            }
            std::fill(stop.begin(), stop.end(), 0.0);
            std::fill(sbot.begin(), sbot.end(), 0.0);
            diffuse_pass(1, 2u + (uint32_t)it, sflags, dflux);
            diffuse_pass(0, 2u + (uint32_t)it, sflags, dflux);
            cam_add_scatter();
            iters = it + 1;
            if (q->scatter_tol > 0.0) {
                // Residual of band column c: area-weighted power scattered by this
                // iteration and not yet propagated, over the band's total so far.  It
                // bounds the relative change of the summed flux if the band stops here.
                bool all = true;
                int c = -1;
                for (int bg = 0; bg < Bg; ++bg) {
                    if (!q->band_launch[bg]) continue;
                    ++c;
                    if (!sflags[bg]) continue;
                    double num = 0.0, den = 0.0;
                    for (int p = 0; p < n; ++p) {
                        size_t i = (size_t)p * Bl + c;
                        double sc = stop[i] + sbot[i];
                        num += s->area[p] * sc;
                        den += s->area[p] * (rin[i] + sc);
                    }
                    if (num <= q->scatter_tol * den) conv[bg] = 1;
                    else all = false;
                }
                if (all) break;
            }
        }
    }
    // ---- cameras (RadiationModel.cpp:4358-4616): rendered from the accumulated camera view
    for (int ci = 0; cams && ci < q->ncameras; ++ci) {
        const orc_camera &oc = q->cameras[ci];
        const size_t npx = (size_t)oc.width * oc.height;
        std::vector<double> pix(npx * Bl, 0.0);
        std::vector<uint32_t> lab(npx, 0u);
        std::vector<float> dep(npx, 0.f);
        if (scattering && (emission || diffuse || rundirect)) {
            Cam c;
            c.pos = v3(oc.position[0], oc.position[1], oc.position[2]);
            camera_rotation(oc.direction[0], oc.direction[1], c.M);
            c.focal = oc.focal_length;
            c.lens = oc.lens_diameter;
            c.inv_aspect = 1.0f / oc.fov_aspect;
            c.L = oc.viewplane_length;
            c.W = oc.width;
            c.H = oc.height;
            c.aa = std::max(oc.antialiasing, 1);
            c.seed = oc.seed;
            c.id = oc.camera_id;
            std::vector<float> rt(ctop.size()), rb(cbot.size());
            for (size_t i = 0; i < ctop.size(); ++i) {
                rt[i] = (float)ctop[i];
                rb[i] = (float)cbot[i];
            }
            CamSky sky;
            sky.sky_radiance = q->cam_sky_radiance;
            sky.disk_radiance = q->cam_disk_radiance;
            sky.diffuse_flux = q->cam_diffuse_flux;
            sky.prague = q->cam_prague;
            sky.emission = q->cam_emission;
            sky.sun = v3(q->cam_sun[0], q->cam_sun[1], q->cam_sun[2]);
            sky.disk_cos = q->cam_disk_cos;
            render_camera(*s, c, Bl, src, q->source_flux, rt.data(), rb.data(), sky, pix.data(), lab.data(), dep.data());
        }
        if (oc.pixels)
            for (size_t i = 0; i < pix.size(); ++i) oc.pixels[i] = (float)pix[i];
        if (oc.labels) std::copy(lab.begin(), lab.end(), oc.labels);
        if (oc.depths) std::copy(dep.begin(), dep.end(), oc.depths);
    }
    for (size_t i = 0; i < (size_t)n * Bl; ++i) flux_out[i] = rin[i] + stop[i] + sbot[i];
    if (stats) {
        stats[0] = n_rays;
        stats[1] = n_nodes;
        stats[2] = n_prims;
        stats[3] = n_hits;
        stats[4] = (uint64_t)iters;
    }
    return 0;
}

}  // extern "C"
