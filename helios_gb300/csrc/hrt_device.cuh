// hrt_device.cuh -- device-side building blocks of the GB300 radiation engine.
//
// Arithmetic contract: all FP32 geometry (ray generation, primitive records,
// bounding boxes, Morton codes, slab and primitive tests) is written as plain
// IEEE-754 single-precision +, -, *, / and sqrt sequences and this library is
// compiled with --fmad=false (no contraction), -prec-div=true and
// -prec-sqrt=true.  The same sequences evaluated on the host give bit-identical
// results, which is what lets the device LBVH be checked bit-for-bit against a
// host build and lets hit IDs be compared exactly.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace hrt {

// Primitive type codes (RayTracingTypes.h:45 of the reference radiation plugin).
enum : uint32_t { PT_PATCH = 0, PT_TRI = 1, PT_DISK = 2, PT_TILE = 3, PT_VOXEL = 4, PT_BBOX = 5 };

// Error bits of the per-context device status word.
enum : uint32_t { ERR_STACK = 1u, ERR_WRAP = 2u, ERR_TIMEOUT = 4u, ERR_BOUNDS = 8u, ERR_BUDGET = 16u };

constexpr int kStack = 64;           // traversal stack entries per ray
constexpr int32_t kEmptyChild = ~0x7FFFFFFF;

struct f3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 scl(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ f3 normalize(f3 a) {
    float l = sqrtf(dot(a, a));
    return mk(a.x / l, a.y / l, a.z / l);
}
__device__ __forceinline__ float get(f3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
__device__ __forceinline__ f3 xyz(float4 v) { return mk(v.x, v.y, v.z); }

// T . (px, py, 0, 1) for a row-major 4x4 transform.
__device__ __forceinline__ f3 xform(const float *T, float px, float py) {
    return mk((T[0] * px + T[1] * py) + T[3], (T[4] * px + T[5] * py) + T[7],
              (T[8] * px + T[9] * py) + T[11]);
}

// ------------------------------------------------------------------ Philox ---
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
struct u4 {
    uint32_t a, b, c, d;
};
__device__ __forceinline__ u4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                     uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    return u4{c0, c1, c2, c3};
}
__device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// cos(2*pi*u), sin(2*pi*u) for u in [0,1): reduction to [0, pi/4] and Taylor
// polynomials (coefficients 1/k!) evaluated in a fixed order.
__device__ __forceinline__ void sincos2pi(float u, float *c_out, float *s_out) {
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

// Natural logarithm of x in (0, 1] for the voxel free-path draw: x = m * 2^e with m in
// [sqrt(1/2), sqrt(2)), ln m = 2 atanh(z), z = (m - 1) / (m + 1), Taylor series to z^9
// (|z| <= 0.172; truncation below 1e-9).  Plain single-precision steps, so the host
// restatement gives the same bits.
__device__ __forceinline__ float ln_unit(float x) {
    uint32_t b = __float_as_uint(x);
    int e = (int)((b >> 23) & 0xFFu) - 127;
    float m = __uint_as_float((b & 0x7FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e = e + 1;
    }
    float z = (m - 1.0f) / (m + 1.0f);
    float z2 = z * z;
    float s = 1.0f + z2 * (0.333333333f + z2 * (0.2f + z2 * (0.142857143f + z2 * 0.111111111f)));
    return (float)e * 0.693147181f + 2.0f * z * s;
}

// Concentric square-to-disk map (Shirley & Chiu, JGT 1997) of (u, v) in [0,1)^2.
__device__ __forceinline__ void concentric(float u, float v, float *x, float *y) {
    float sx = -1.0f + 2.0f * u, sy = -1.0f + 2.0f * v;
    float r, ph;  // ph in units of pi/4
    if (sx > -sy) {
        if (sx > sy) {
            r = sx;
            ph = sy / sx;
        } else {
            r = sy;
            ph = 2.0f - sx / sy;
        }
    } else {
        if (sx < sy) {
            r = -sx;
            ph = 4.0f + sy / sx;
        } else {
            r = -sy;
            ph = (sy != 0.f) ? 6.0f - sx / sy : 0.f;
        }
    }
    float frac = ph * 0.125f;
    if (frac < 0.f) frac = frac + 1.0f;
    float c, s;
    sincos2pi(frac, &c, &s);
    *x = r * c;
    *y = r * s;
}

// Orthonormal basis about unit n (Duff et al., JCGT 6(1), 2017).
__device__ __forceinline__ void onb(f3 n, f3 *t1, f3 *t2) {
    float sign = copysignf(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    *t1 = mk(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    *t2 = mk(b, sign + n.y * n.y * a, -n.y);
}

// Cosine-weighted stratified direction about n (stratum (ti, pi) of dimx x dimy).
__device__ __forceinline__ f3 diffuse_dir(f3 n, int ti, int pi, int dimx, int dimy, float j0, float j1) {
    float Rt = ((float)ti + j0) / (float)dimx;
    float Rp = ((float)pi + j1) / (float)dimy;
    float st = sqrtf(Rt);
    float ct = sqrtf(1.0f - Rt);
    float cp, sp;
    sincos2pi(Rp, &cp, &sp);
    float lx = st * cp, ly = st * sp;
    f3 t1, t2;
    onb(n, &t1, &t2);
    return mk((t1.x * lx + t2.x * ly) + n.x * ct, (t1.y * lx + t2.y * ly) + n.y * ct,
              (t1.z * lx + t2.z * ly) + n.z * ct);
}

// Voxel leaves scatter isotropically: stratified uniform direction on the upper
// hemisphere (cos theta = 1 - Rt, as OptiX 6 rayGeneration.cu:401-415 samples voxels);
// the bottom-face ray of the same sample flips it, so each pair covers the sphere.
__device__ __forceinline__ f3 voxel_dir(int ti, int pi, int dimx, int dimy, float j0, float j1) {
    float Rt = ((float)ti + j0) / (float)dimx;
    float Rp = ((float)pi + j1) / (float)dimy;
    float ct = 1.0f - Rt;
    float st = sqrtf(fmaxf(0.f, 1.0f - ct * ct));
    float cp, sp;
    sincos2pi(Rp, &cp, &sp);
    return mk(st * cp, st * sp, ct);
}

// Projection coefficient of a voxel's leaves (spherical leaf-angle distribution).
constexpr float kVoxelG = 0.5f;

// Counter words and key of a ray's voxel free-path draws: the draw for voxel v is
// philox(c0, c1, c2 | wrap << 16, v + 1; k0, k1).  It depends on the ray's identity
// and wrap count only, never on traversal order or on how launches are batched.
struct VoxKey {
    uint32_t c0, c1, c2, k0, k1;
};

// ------------------------------------------------------------------ records ---
// Intersection record (64 B, BVH leaf order):
//   r0 = (p0.xyz, type bits)  r1 = (p1.xyz, original index bits)
//   r2 = (p2.xyz, k)          r3 = (p3.xyz, 0)
// patch/bbox: 4 corners; triangle: v0,v1,v2 (r3 = v2); disk: centre, unit normal, (radius,0,0);
// voxel: lo, hi, with k = G * LAD its extinction coefficient (0 for other types).
// Ray-origin record (64 B, original order):
//   g0 = (P.xyz, type bits) g1 = (A.xyz, twosided bits) g2 = (B.xyz, 0) g3 = (N.xyz, 0)
// with sample point P + u*A + v*B and unit normal N (disk: P = centre, unit disk over A, B;
// voxel: P = lower corner, g3 = third edge C, point P + u*A + v*B + w*C).

__device__ __forceinline__ void make_records(const float *T, uint32_t type, float lad, float4 rec[4], float4 g[4],
                                             f3 *lo, f3 *hi) {
    f3 p0, p1, p2, p3;
    uint32_t rt = type;
    if (type == PT_TRI) {
        p0 = xform(T, 0.f, 0.f);
        p1 = xform(T, 0.f, 1.f);
        p2 = xform(T, 1.f, 1.f);
        p3 = p2;
    } else if (type == PT_DISK) {
        p0 = xform(T, 0.f, 0.f);
        f3 ax = mk(T[0], T[4], T[8]), ay = mk(T[1], T[5], T[9]);
        p1 = normalize(cross(ax, ay));
        p2 = mk(sqrtf(dot(ax, ax)), 0.f, 0.f);
        p3 = p0;
    } else if (type == PT_VOXEL) {
        f3 c = mk(T[3], T[7], T[11]);
        f3 h = mk(fabsf(T[0]) * 0.5f, fabsf(T[5]) * 0.5f, fabsf(T[10]) * 0.5f);
        p0 = sub(c, h);
        p1 = add(c, h);
        p2 = p0;
        p3 = p1;
    } else {
        rt = PT_PATCH;
        p0 = xform(T, -0.5f, -0.5f);
        p1 = xform(T, 0.5f, -0.5f);
        p2 = xform(T, 0.5f, 0.5f);
        p3 = xform(T, -0.5f, 0.5f);
    }
    rec[0] = make_float4(p0.x, p0.y, p0.z, __uint_as_float(rt));
    rec[1] = make_float4(p1.x, p1.y, p1.z, 0.f);
    rec[2] = make_float4(p2.x, p2.y, p2.z, (rt == PT_VOXEL) ? kVoxelG * lad : 0.f);
    rec[3] = make_float4(p3.x, p3.y, p3.z, 0.f);
    // bounds
    if (rt == PT_DISK) {
        float rad = p2.x;
        f3 n = p1;
        float ex = rad * sqrtf(fmaxf(0.f, 1.0f - n.x * n.x));
        float ey = rad * sqrtf(fmaxf(0.f, 1.0f - n.y * n.y));
        float ez = rad * sqrtf(fmaxf(0.f, 1.0f - n.z * n.z));
        *lo = mk(p0.x - ex, p0.y - ey, p0.z - ez);
        *hi = mk(p0.x + ex, p0.y + ey, p0.z + ez);
    } else {
        f3 v[4] = {p0, p1, p2, p3};
        int nv = (rt == PT_TRI) ? 3 : (rt == PT_VOXEL ? 2 : 4);
        f3 a = v[0], b = v[0];
        for (int i = 1; i < nv; ++i) {
            a = mk(fminf(a.x, v[i].x), fminf(a.y, v[i].y), fminf(a.z, v[i].z));
            b = mk(fmaxf(b.x, v[i].x), fmaxf(b.y, v[i].y), fmaxf(b.z, v[i].z));
        }
        *lo = a;
        *hi = b;
    }
    // origin-sampling record
    f3 A = mk(T[0], T[4], T[8]), B = mk(T[1], T[5], T[9]), P, N;
    if (type == PT_TRI) {
        P = mk(T[3], T[7], T[11]);
        N = normalize(cross(B, A));
    } else if (type == PT_DISK) {
        P = mk(T[3], T[7], T[11]);
        N = normalize(cross(A, B));
    } else if (type == PT_VOXEL) {
        N = mk(T[2], T[6], T[10]);
        P = mk(((T[0] * -0.5f + T[1] * -0.5f) + T[2] * -0.5f) + T[3],
               ((T[4] * -0.5f + T[5] * -0.5f) + T[6] * -0.5f) + T[7],
               ((T[8] * -0.5f + T[9] * -0.5f) + T[10] * -0.5f) + T[11]);
    } else {
        P = xform(T, -0.5f, -0.5f);
        N = normalize(cross(A, B));
    }
    g[0] = make_float4(P.x, P.y, P.z, __uint_as_float(type));
    g[1] = make_float4(A.x, A.y, A.z, 0.f);
    g[2] = make_float4(B.x, B.y, B.z, 0.f);
    g[3] = make_float4(N.x, N.y, N.z, 0.f);
}

// Ray origin from uniform numbers u, v (w: voxels only).  Disks use the concentric map
// (OptiX 6 rayGeneration.cu:346-390), voxels the whole box (rayGeneration.cu:392-397).
__device__ __forceinline__ f3 sample_point(const float4 g[4], uint32_t type, float u, float v, float w) {
    f3 P = xyz(g[0]), A = xyz(g[1]), B = xyz(g[2]);
    if (type == PT_TRI) {
        float a = u < v ? u : v, b = u < v ? v : u;
        return mk((P.x + a * A.x) + b * B.x, (P.y + a * A.y) + b * B.y, (P.z + a * A.z) + b * B.z);
    }
    if (type == PT_DISK) {
        float x, y;
        concentric(u, v, &x, &y);
        return mk((P.x + x * A.x) + y * B.x, (P.y + x * A.y) + y * B.y, (P.z + x * A.z) + y * B.z);
    }
    if (type == PT_VOXEL) {
        f3 C = xyz(g[3]);
        return mk(((P.x + u * A.x) + v * B.x) + w * C.x, ((P.y + u * A.y) + v * B.y) + w * C.y,
                  ((P.z + u * A.z) + v * B.z) + w * C.z);
    }
    return mk((P.x + u * A.x) + v * B.x, (P.y + u * A.y) + v * B.y, (P.z + u * A.z) + v * B.z);
}

// ------------------------------------------------------- compressed 4-wide BVH ---
// Node (64 B, two 256-bit loads):
//   q0 = (px, py, pz, sx)       origin p (the node box's lower corner) and the x step
//   q1 = (lox, loy, loz, hix)   quantised child boxes, byte k = child k (0 <= q <= 255)
//   q2 = (hiy, hiz, c0, c1)     child refs c_k: >= 0 node, ~slot leaf, kEmptyChild none
//   q3 = (c2, c3, sy, sz)       the y and z steps
// Each step s = 2^(e - 127) is a power of two (e in [1, 254]), stored as a float so that the
// test reads it without decoding.
// An empty child slot has lo bytes 255 and hi bytes 0: an inverted box that no ray enters.
// On every axis the slab slope a = inv * s is nonzero (|inv| >= 1 for a unit direction,
// s >= 2^-126), so the near plane lies beyond the far plane; an infinite slope gives a NaN
// plane, which the min/max skip, and an infinite near or far plane, which fails the test.
// Child k's box per axis: [p + lo_k * s, p + hi_k * s] in FP32 (q * s is exact; one rounded
// add).  The build picks the bytes so that these values enclose the child's FP32 box (itself
// padded), so a slab test on the decoded box never culls an accepted hit (after Ylitie,
// Karras, Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs",
// HPG 2017, with 4 children per node).
__device__ __forceinline__ float q_step(uint32_t e) { return __uint_as_float(e << 23); }

// Unsigned 32-bit division by a divisor fixed for a launch, by multiplication (Granlund and
// Montgomery, "Division by invariant integers using multiplication", PLDI 1994, the round-up
// method with a 32-bit multiplier): with l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1,
// n / d = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0) for t = umulhi(m, n), exactly for every
// 32-bit n and 1 <= d < 2^32.
struct FastDiv {
    uint32_t m, s1, s2;
};
__host__ __device__ __forceinline__ FastDiv make_fastdiv(uint32_t d) {
    uint32_t l = 0;
    while (l < 32 && (1ull << l) < d) ++l;
    FastDiv f;
    f.m = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    f.s1 = l < 1 ? l : 1;
    f.s2 = l > 1 ? l - 1 : 0;
    return f;
}
__host__ __device__ __forceinline__ uint32_t fast_div(uint32_t n, const FastDiv &f) {
    const uint32_t t = (uint32_t)(((uint64_t)f.m * n) >> 32);  // umulhi
    return (t + ((n - t) >> f.s1)) >> f.s2;
}
// The four float4 of a 64-byte node (binary or 4-wide) in two 256-bit read-only loads; node
// arrays start on a 256-byte boundary, so every node is 64-byte aligned.
__device__ __forceinline__ void load_node64(const float4 *nodes, int32_t i, float4 &q0, float4 &q1, float4 &q2,
                                           float4 &q3) {
    const float4 *a = nodes + 4 * (size_t)i;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(q0.x), "=f"(q0.y), "=f"(q0.z), "=f"(q0.w), "=f"(q1.x), "=f"(q1.y), "=f"(q1.z), "=f"(q1.w)
        : "l"(a));
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(q2.x), "=f"(q2.y), "=f"(q2.z), "=f"(q2.w), "=f"(q3.x), "=f"(q3.y), "=f"(q3.z), "=f"(q3.w)
        : "l"(a + 2));
}
__device__ __forceinline__ float q_decode(float p, uint32_t q, float s) { return p + (float)q * s; }
__device__ __forceinline__ uint32_t q_byte(uint32_t w, int k) { return (w >> (8 * k)) & 0xFFu; }
// Three-input minimum / maximum (PTX min.f32 / max.f32 with three sources; a NaN input
// is ignored, as by fminf / fmaxf).
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
// Byte k of w as an exact float: one byte permute builds 0x4B0000qq = 2^23 + q.
__device__ __forceinline__ float q_float(uint32_t w, int k) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, (uint32_t)k | 0x7540u)) - 8388608.0f;
}

// Packed FP32 pairs (PTX .f32x2 on sm_100 and later): one instruction applies the same
// IEEE operation (round to nearest) to both halves of a 64-bit register pair.
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(unsigned long long r, float *lo, float *hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(*lo), "=f"(*hi) : "l"(r));
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b, unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// Byte k of w as the float 2^23 + q (q_float before its subtraction).
__device__ __forceinline__ float q_biased(uint32_t w, int k) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, (uint32_t)k | 0x7540u));
}

// Leaf-box padding: each face moves out by (|x| + extent) * 2^-20.
__device__ __forceinline__ float pad_lo(float x, float ext) { return x - (fabsf(x) + ext) * 9.5367431640625e-07f; }
__device__ __forceinline__ float pad_hi(float x, float ext) { return x + (fabsf(x) + ext) * 9.5367431640625e-07f; }

// ------------------------------------------------------------------ tests ---
struct WT {
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
__device__ __forceinline__ WT wt_setup(f3 d) {
    WT w;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    w.kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    w.kx = (w.kz == 2) ? 0 : w.kz + 1;
    w.ky = (w.kx == 2) ? 0 : w.kx + 1;
    float dz = get(d, w.kz);
    if (dz < 0.f) {
        int t = w.kx;
        w.kx = w.ky;
        w.ky = t;
    }
    w.Sx = get(d, w.kx) / dz;
    w.Sy = get(d, w.ky) / dz;
    w.Sz = 1.0f / dz;
    return w;
}

__device__ __forceinline__ float edgef(float px, float py, float qx, float qy) {
    float e = px * qy - py * qx;
    if (e == 0.f) e = (float)((double)px * (double)qy - (double)py * (double)qx);
    return e;
}

// Watertight polygon test (Woop, Benthin, Wald, JCGT 2(1), 2013) for triangles (n=3)
// and planar convex quads (n=4).  face = 1 when dot(d, n) < 0.
template <int NV>
__device__ __forceinline__ bool poly_hit(const WT &w, f3 o, float tmin, const f3 *v, float tmax, float *t_out,
                                         int *face_out) {
    float px[NV], py[NV], pz[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        f3 a = sub(v[i], o);
        float az = get(a, w.kz);
        px[i] = get(a, w.kx) - w.Sx * az;
        py[i] = get(a, w.ky) - w.Sy * az;
        pz[i] = w.Sz * az;
    }
    float e[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        int j = (i + 1 == NV) ? 0 : i + 1;
        e[i] = edgef(px[i], py[i], px[j], py[j]);
    }
    bool anyneg = false, anypos = false;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        anyneg = anyneg || (e[i] < 0.f);
        anypos = anypos || (e[i] > 0.f);
    }
    if (anyneg && anypos) return false;
    float e20 = (NV == 3) ? e[NV - 1] : edgef(px[2], py[2], px[0], py[0]);
    float det = (e[1] + e20) + e[0];
    if (det == 0.f) return false;
    float T = (e[1] * pz[0] + e20 * pz[1]) + e[0] * pz[2];
    float t = T / det;
    if (!(t >= tmin) || !(t <= tmax)) return false;
    *t_out = t;
    // det < 0 <=> dot(d, n) < 0 for n = (v1-v0) x (v2-v0): the ray meets the top face
    *face_out = (det < 0.f) ? 1 : 0;
    return true;
}

__device__ __forceinline__ float safe_inv(float d) {
    if (fabsf(d) < 1e-30f) d = copysignf(1e-30f, d);
    return 1.0f / d;
}

__device__ __forceinline__ bool slab(f3 o, f3 inv, f3 lo, f3 hi, float tmin, float tmax, float *tnear) {
    float t0x = (lo.x - o.x) * inv.x, t1x = (hi.x - o.x) * inv.x;
    float t0y = (lo.y - o.y) * inv.y, t1y = (hi.y - o.y) * inv.y;
    float t0z = (lo.z - o.z) * inv.z, t1z = (hi.z - o.z) * inv.z;
    float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
    float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax));
    *tnear = tn;
    return tn <= tf;
}

// Slab test for BVH node boxes with the ray's origin pre-multiplied (ooi = o * inv):
// t = lo * inv - ooi in one fused multiply-add per plane.  Node boxes are padded, so
// the rounding of ooi never culls a box that holds an accepted hit.
__device__ __forceinline__ bool slab_node(f3 ooi, f3 inv, f3 lo, f3 hi, float tmin, float tmax, float *tnear) {
    float t0x = __fmaf_rn(lo.x, inv.x, -ooi.x), t1x = __fmaf_rn(hi.x, inv.x, -ooi.x);
    float t0y = __fmaf_rn(lo.y, inv.y, -ooi.y), t1y = __fmaf_rn(hi.y, inv.y, -ooi.y);
    float t0z = __fmaf_rn(lo.z, inv.z, -ooi.z), t1z = __fmaf_rn(hi.z, inv.z, -ooi.z);
    float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
    float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax));
    *tnear = tn;
    return tn <= tf;
}

// Disk: plane hit inside the radius (reference OptiX 6 primitiveIntersection.cu:236-300).
__device__ __forceinline__ bool disk_hit(f3 o, f3 d, float tmin, f3 c, f3 n, float rad, float tmax, float *t_out,
                                         int *face_out) {
    float nd = dot(d, n);
    if (nd == 0.f) return false;
    float t = dot(sub(c, o), n) / nd;
    if (!(t >= tmin) || !(t <= tmax)) return false;
    f3 h = sub(add(o, scl(d, t)), c);
    if (dot(h, h) > rad * rad) return false;
    *t_out = t;
    *face_out = (nd < 0.f) ? 1 : 0;
    return true;
}

// Voxel: a turbid medium with extinction k = G * LAD.  The reference defines no voxel
// physics (its OptiX 6 absorption is commented out, rayHit.cu:278-290), so this engine
// does: the ray's path through the box, from max(entry, tmin) to the exit, is
// intercepted at the free path s = -ln(xi) / k with xi in (0, 1] drawn per (ray, voxel,
// wrap).  A ray starting inside the box crosses the rest of it.  The hit face is the top.
__device__ __forceinline__ bool voxel_hit(f3 o, f3 inv, float tmin, f3 lo, f3 hi, float k, float tmax,
                                          const VoxKey &vk, uint32_t vid, float *t_out, int *face_out) {
    if (!(k > 0.f)) return false;
    float t0x = (lo.x - o.x) * inv.x, t1x = (hi.x - o.x) * inv.x;
    float t0y = (lo.y - o.y) * inv.y, t1y = (hi.y - o.y) * inv.y;
    float t0z = (lo.z - o.z) * inv.z, t1z = (hi.z - o.z) * inv.z;
    float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
    float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    if (!(tn < tf)) return false;
    u4 u = philox(vk.c0, vk.c1, vk.c2, vid + 1u, vk.k0, vk.k1);
    float t = tn + -ln_unit(1.0f - u01(u.a)) / k;
    if (!(t < tf) || !(t <= tmax)) return false;
    *t_out = t;
    *face_out = 1;
    return true;
}

// ---------------------------------------------------------------- texture masks ---
// A masked patch or triangle is hit only where its mask texel is opaque (reference
// OptiX8DeviceCode.cu:173-187, 397-416, 457-476); origins avoid transparent texels.
struct MaskSet {
    const int32_t *id;       // [n] mask of each primitive (original order, -1 none); null: no masks
    const int32_t *uv_id;    // [n] >= 0: uv holds the primitive's texture coordinates
    const float *uv;         // [n*8] corner (u,v) pairs
    const int32_t *size;     // [nmasks*2] width, height
    const uint32_t *offset;  // [nmasks] start of each mask in data
    const uint8_t *data;     // row-major texels, nonzero = opaque
    const float *T;          // [n*16] transforms (original order)
};

__device__ __forceinline__ bool mask_opaque(const MaskSet &m, int id, float u, float v) {
    const int w = m.size[2 * id], h = m.size[2 * id + 1];
    int ix = (int)floorf((float)(w - 1) * u);
    int iy = (int)floorf((float)(h - 1) * (1.0f - v));
    ix = ix < 0 ? 0 : (ix > w - 1 ? w - 1 : ix);
    iy = iy < 0 ? 0 : (iy > h - 1 ? h - 1 : iy);
    return m.data[m.offset[id] + (uint32_t)(iy * w + ix)] != 0;
}

// texture (u, v) of patch p at local coordinates (lu, lv) in [-0.5, 0.5]^2
__device__ __forceinline__ void patch_uv(const MaskSet &m, uint32_t p, float lu, float lv, float *uu, float *vv) {
    if (m.uv_id[p] >= 0) {
        const float *q = m.uv + 8 * (size_t)p;
        *uu = q[0] + (lu + 0.5f) * (q[2] - q[0]);
        *vv = q[1] + (lv + 0.5f) * (q[5] - q[1]);
    } else {
        *uu = lu + 0.5f;
        *vv = lv + 0.5f;
    }
}

// texture (u, v) of triangle p at barycentrics beta (vertex 1) and gamma (vertex 2)
__device__ __forceinline__ void tri_uv(const MaskSet &m, uint32_t p, float beta, float gamma, float *uu, float *vv) {
    if (m.uv_id[p] >= 0) {
        const float *q = m.uv + 8 * (size_t)p;
        *uu = (q[0] + beta * (q[2] - q[0])) + gamma * (q[4] - q[0]);
        *vv = 1.0f - ((q[1] + beta * (q[3] - q[1])) + gamma * (q[5] - q[1]));
    } else {
        *uu = beta + gamma;
        *vv = gamma;
    }
}

// Is the geometric hit at distance t on masked primitive p on an opaque texel?  Patches
// use the local coordinates of the hit point, triangles the Cramer barycentrics.
static __device__ __noinline__ bool mask_hit_opaque(const MaskSet &m, uint32_t p, uint32_t type, f3 o, f3 d, float t) {
    const float *T = m.T + 16 * (size_t)p;
    float uu, vv;
    if (type == PT_TRI) {
        const f3 v0 = mk(T[3], T[7], T[11]), v1 = xform(T, 0.f, 1.f), v2 = xform(T, 1.f, 1.f);
        const float a = v0.x - v1.x, b = v0.x - v2.x, c = d.x, dd = v0.x - o.x;
        const float e = v0.y - v1.y, f = v0.y - v2.y, g = d.y, h = v0.y - o.y;
        const float i = v0.z - v1.z, j = v0.z - v2.z, k = d.z, l = v0.z - o.z;
        const float mm = f * k - g * j, nn = h * k - g * l, pp = f * l - h * j;
        const float q = g * i - e * k, sq = e * j - f * i;
        const float den = a * mm + b * q + c * sq;
        if (den == 0.f) return true;
        const float iv = 1.f / den;
        const float beta = (dd * mm - b * nn - c * pp) * iv;
        const float r = e * l - h * i;
        const float gamma = (a * nn + dd * q + c * r) * iv;
        tri_uv(m, p, beta, gamma, &uu, &vv);
    } else {
        const f3 hl = sub(add(o, scl(d, t)), mk(T[3], T[7], T[11]));
        const f3 lx = mk(T[0], T[4], T[8]), ly = mk(T[1], T[5], T[9]);
        const float lu = dot(hl, lx) / dot(lx, lx), lv = dot(hl, ly) / dot(ly, ly);
        patch_uv(m, p, lu, lv, &uu, &vv);
    }
    return mask_opaque(m, m.id[p], uu, vv);
}

// Test record `slot`; on success returns t, face and the original primitive index.
// Transmittance, reflectance and absorptance of one dielectric sheet (a translucent cover)
// of refractive index n and absorption product K*L at incidence cosine c: Fresnel
// reflection r at each face (s and p polarisation averaged), Bouguer attenuation ta along
// the refracted path, incoherent multiple reflections T = ta (1-r)^2 / (1 - (r ta)^2),
// R = r (1 + ta T).  The physics and clamps of the reference's glass_tau_rho_alpha
// (OptiX8DeviceCode.cu:90-134), written in cosines (no trigonometric calls).
__device__ __forceinline__ void glass_trs(float c, float n, float KL, float *tau, float *rho, float *alpha) {
    c = fminf(1.f, fmaxf(1e-4f, c));
    const float st = sqrtf(fmaxf(0.f, 1.f - c * c)) / n;
    const float ct = sqrtf(fmaxf(0.f, 1.f - st * st));
    const float as = (c - n * ct) / (c + n * ct);
    const float ap = (n * c - ct) / (n * c + ct);
    const float ta = KL > 0.f ? expf(-KL / fmaxf(1e-4f, ct)) : 1.f;
    float T = 0.f, R = 0.f;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float r = k == 0 ? as * as : ap * ap;
        const float q = r * ta;
        const float den = fmaxf(1e-6f, 1.f - q * q);
        const float ti = ta * (1.f - r) * (1.f - r) / den;
        const float ri = r * (1.f + ta * ti);
        T += 0.5f * ti;
        R += 0.5f * ri;
    }
    T = fmaxf(0.f, fminf(1.f, T));
    R = fmaxf(0.f, fminf(1.f, R));
    *tau = T;
    *rho = R;
    *alpha = fmaxf(0.f, 1.f - T - R);
}

// VOX = false leaves voxels out (for scenes known to hold none).
template <bool VOX = true>
__device__ __forceinline__ bool rec_hit(const float4 *__restrict__ rec, uint32_t slot, const WT &w, f3 o, f3 d,
                                        f3 inv, float tmin, float tmax, const VoxKey &vk, float *t, int *face,
                                        uint32_t *orig, const MaskSet &ms) {
    const float4 *r = rec + 4 * (size_t)slot;
    float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2);
    uint32_t type = __float_as_uint(r0.w);
    *orig = __float_as_uint(r1.w);
    bool ok;
    if (type == PT_TRI) {
        f3 v[3] = {xyz(r0), xyz(r1), xyz(r2)};
        ok = poly_hit<3>(w, o, tmin, v, tmax, t, face);
    } else if (type == PT_PATCH) {
        float4 r3 = __ldg(r + 3);
        f3 v[4] = {xyz(r0), xyz(r1), xyz(r2), xyz(r3)};
        ok = poly_hit<4>(w, o, tmin, v, tmax, t, face);
    } else if (type == PT_DISK) {
        ok = disk_hit(o, d, tmin, xyz(r0), xyz(r1), r2.x, tmax, t, face);
    } else if (VOX && type == PT_VOXEL) {
        ok = voxel_hit(o, inv, tmin, xyz(r0), xyz(r1), r2.w, tmax, vk, *orig, t, face);
    } else {
        ok = false;
    }
    if (ok && ms.id && (type == PT_TRI || type == PT_PATCH) && ms.id[*orig] >= 0)
        ok = mask_hit_opaque(ms, *orig, type, o, d, *t);
    return ok;
}

}  // namespace hrt
