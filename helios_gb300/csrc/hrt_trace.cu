// hrt_trace.cu -- ray generation, BVH traversal and per-primitive accumulation.
//
// Replaces the reference's OptiX device programs
// (plugins/radiation/src/optix8/OptiX8DeviceCode.cu):
//   __raygen__direct  :1210-1465  -> k_direct   (+ __miss__direct :514-596 via the epilogue)
//   __raygen__diffuse :1471-1658  -> k_diffuse  (+ __closesthit__diffuse :930-1001,
//                                                 __miss__diffuse :598-671)
//   __intersection__patch :320-490 -> rec_hit (watertight; hrt_device.cuh)
// Every deposit of the reference lands on the ray's ORIGIN primitive, so a ray
// only produces a value for its origin.  Rays are numbered so that the rays of
// one primitive are consecutive; a warp therefore holds the rays of one or two
// primitives and reduces their values with a segmented shuffle scan in FP64
// before one atomic per (primitive, band) segment.  Material factors
// (1-rho-tau, rho, tau) are applied afterwards per primitive (epilogues), which
// equals the reference's per-ray products in exact arithmetic.
#include <cstdlib>

#include "hrt_device.cuh"
#include "hrt_internal.h"

namespace hrt {

namespace {

constexpr int kBlock = 256;

struct Hit {
    float t;
    uint32_t prim;  // original index, 0xFFFFFFFF = miss, kLost = dropped after the wrap limit
    int face;
};
constexpr uint32_t kLost = 0xFFFFFFFEu;

__device__ __forceinline__ void raise(uint32_t *status, uint32_t bit) {
    if (status) atomicOr(status, bit);
}

// Closest (or any) hit over the BVH.  Visiting order: both child boxes are
// tested against the current best distance; leaf children are intersected at
// once; of two internal children the nearer is entered and the farther pushed.
template <bool STATS>
__device__ Hit trace_bvh(const TraceScene &sc, f3 o, f3 d, float tmin, float tmax, bool anyhit, const VoxKey &vk,
                         uint32_t *nv, uint32_t *np) {
    Hit h{tmax, 0xFFFFFFFFu, 0};
    if (sc.n == 0) return h;
    WT w = wt_setup(d);
    f3 inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    f3 ooi = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
    int32_t stack[kStack];
    int sp = 0;
    int32_t cur = 0;
    float best = tmax;
    const uint32_t ni = (uint32_t)(sc.n > 1 ? sc.n - 1 : 1);
    uint32_t budget = 2u * (uint32_t)sc.n + 64u;  // a ray visits each node at most once
    for (;;) {
        if ((uint32_t)cur >= ni || budget-- == 0u) {
            raise(sc.status, ERR_BOUNDS);
            return h;
        }
        if (STATS) ++*nv;
        const float4 *nd = sc.nodes + 4 * (size_t)cur;
        float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3);
        int32_t c[2] = {__float_as_int(n3.x), __float_as_int(n3.y)};
        float tn0, tn1;
        bool hb[2];
        hb[0] = slab_node(ooi, inv, mk(n0.x, n0.y, n0.z), mk(n0.w, n1.x, n1.y), tmin, best, &tn0);
        hb[1] = slab_node(ooi, inv, mk(n1.z, n1.w, n2.x), mk(n2.y, n2.z, n2.w), tmin, best, &tn1);
        int32_t next[2];
        int nn = 0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (!hb[k]) continue;
            int32_t ck = c[k];
            if (ck < 0) {
                if (ck == kEmptyChild) continue;
                if ((uint32_t)(~ck) >= (uint32_t)sc.n) {
                    raise(sc.status, ERR_BOUNDS);
                    continue;
                }
                float t;
                int face;
                uint32_t orig;
                if (STATS) ++*np;
                if (rec_hit(sc.rec, (uint32_t)(~ck), w, o, d, inv, tmin, best, vk, &t, &face, &orig)) {
                    if (h.prim == 0xFFFFFFFFu || t < h.t || (t == h.t && orig < h.prim)) {
                        h.t = t;
                        h.prim = orig;
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
            bool sw = tn1 < tn0;
            int32_t nearc = sw ? next[1] : next[0];
            int32_t farc = sw ? next[0] : next[1];
            if (sp >= kStack) {
                raise(sc.status, ERR_STACK);
                return h;
            }
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

// Periodic walls: closest wall before `lim`.
__device__ __forceinline__ bool wall_closest(const TraceScene &sc, f3 o, f3 d, float tmin, float lim, float *tb,
                                             int *which) {
    WT w = wt_setup(d);
    bool any = false;
    float best = lim;
    for (int b = 0; b < sc.nbbox; ++b) {
        f3 v[4] = {xyz(sc.bbox[4 * b]), xyz(sc.bbox[4 * b + 1]), xyz(sc.bbox[4 * b + 2]), xyz(sc.bbox[4 * b + 3])};
        float t;
        int face;
        if (poly_hit<4>(w, o, tmin, v, best, &t, &face)) {
            if (!any || t < best) {
                best = t;
                *which = b;
                any = true;
            }
        }
    }
    *tb = best;
    return any;
}

// Trace with periodic wrapping (<= 10 wraps; OptiX8DeviceCode.cu:763-789, 1440-1459).
template <bool STATS>
__device__ Hit trace_full(const TraceScene &sc, f3 o, f3 d, float tmin, float tmax, bool anyhit, VoxKey vk,
                          uint32_t *nv, uint32_t *np) {
    const uint32_t c2 = vk.c2;
    for (int wrap = 0; wrap < 10; ++wrap) {
        vk.c2 = c2 | ((uint32_t)wrap << 16);
        Hit h = trace_bvh<STATS>(sc, o, d, tmin, tmax, anyhit && sc.nbbox == 0, vk, nv, np);
        if (sc.nbbox == 0) return h;
        float tb;
        int which = -1;
        float lim = (h.prim != 0xFFFFFFFFu) ? h.t : tmax;
        if (!wall_closest(sc, o, d, tmin, lim, &tb, &which) || (h.prim != 0xFFFFFFFFu && !(tb < h.t))) return h;
        f3 hp = add(o, scl(d, tb));
        bool xwall = (sc.periodic_x == 1.f) && which < 2;
        if (xwall) {
            float width = sc.bbox[4].x - sc.bbox[0].x;
            hp.x = hp.x + ((which == 0) ? width : -width);
        } else {
            int yb = (sc.periodic_x == 1.f) ? 2 : 0;
            float width = sc.bbox[4 * (yb + 1)].y - sc.bbox[4 * yb].y;
            hp.y = hp.y + ((which == yb) ? width : -width);
        }
        o = hp;
    }
    // The tenth trace ended on a wall again: the reference's loop stops there and no
    // miss or closest-hit program deposits anything for this ray.
    return Hit{tmax, kLost, 0};
}

__device__ __forceinline__ void load_rgen(const TraceScene &sc, uint32_t p, float4 g[4]) {
    const float4 *s = sc.rgen + 4 * (size_t)p;
    g[0] = __ldg(s);
    g[1] = __ldg(s + 1);
    g[2] = __ldg(s + 2);
    g[3] = __ldg(s + 3);
}

__device__ __forceinline__ void count_visits(const TraceScene &sc, uint32_t nv, uint32_t np) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        nv += __shfl_down_sync(0xffffffffu, nv, d);
        np += __shfl_down_sync(0xffffffffu, np, d);
    }
    if ((threadIdx.x & 31) == 0 && sc.visits) {
        atomicAdd(sc.visits, (unsigned long long)nv);
        atomicAdd(sc.visits + 1, (unsigned long long)np);
    }
}

__device__ __forceinline__ void count_rays(const TraceScene &sc, bool traced) {
    unsigned m = __ballot_sync(0xffffffffu, traced);
    if ((threadIdx.x & 31) == 0 && m && sc.rays) atomicAdd(sc.rays, (unsigned long long)__popc(m));
}

// Segmented warp sum over consecutive lanes with equal key; the last lane of
// each segment adds the segment total to dst[key*stride + j].  All 32 lanes
// must call this (inactive lanes pass key = 0xFFFFFFFF).
template <int NV>
__device__ __forceinline__ void warp_segment_add(uint32_t key, double (&v)[NV], int nv, double *dst, int stride) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int dlt = 1; dlt < 32; dlt <<= 1) {
        uint32_t ok = __shfl_up_sync(0xffffffffu, key, dlt);
        bool same = lane >= dlt && ok == key;
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            double y = __shfl_up_sync(0xffffffffu, v[j], dlt);
            if (same) v[j] += y;
        }
    }
    uint32_t nk = __shfl_down_sync(0xffffffffu, key, 1);
    bool tail = (lane == 31) || nk != key;
    if (tail && key != 0xFFFFFFFFu) {
        for (int j = 0; j < nv && j < NV; ++j)
            if (v[j] != 0.0) atomicAdd(dst + (size_t)key * stride + j, v[j]);
    }
}

// ------------------------------------------------------------------ origins --
// Leaf-projection factor of a direct ray's strength: |n . d| on a surface, G on a voxel.
__device__ __forceinline__ double proj(f3 nrm, f3 d, bool vox) {
    return vox ? (double)kVoxelG : (double)fabsf(dot(nrm, d));
}

// Origin of direct ray r of primitive p; u = philox(r, p, c2, 0; seed, pass), c2 =
// source << 1.  Non-triangles are stratified over dimx x dimy cells
// (OptiX8DeviceCode.cu:1270-1290); a voxel's third coordinate uses counter c2 | 1.
__device__ __forceinline__ f3 direct_origin(const float4 g[4], uint32_t type, uint32_t r, uint32_t p, uint32_t c2,
                                            int dimx, int dimy, uint32_t seed, uint32_t pass, const u4 &u) {
    float uu = u01(u.a), vv = u01(u.b), ww = 0.f;
    if (type != PT_TRI) {
        const int xi = (int)(r % (uint32_t)dimx), yi = (int)(r / (uint32_t)dimx);
        uu = ((float)xi + uu) / (float)dimx;
        vv = ((float)yi + vv) / (float)dimy;
    }
    if (type == PT_VOXEL) ww = u01(philox(r, p, c2 | 1u, 0u, seed, pass).a);
    return sample_point(g, type, uu, vv, ww);
}

// Origin and direction of diffuse ray r of primitive p from face `face` (1 top, 0
// bottom).  Surfaces: cosine-weighted about the normal, counter (r, p, face, 0).  Voxels
// (VOX builds only): both faces share the sample of counter (r, p, 1, 0), the third
// coordinate comes from (r, p, 2, 0), and the bottom face flips the direction.
template <bool VOX>
__device__ __forceinline__ void diffuse_ray(const float4 g[4], uint32_t type, uint32_t r, uint32_t p, int face,
                                            int dimx, int dimy, uint32_t seed, uint32_t pass, f3 *org, f3 *dir) {
    const int ti = (int)(r % (uint32_t)dimx), pi = (int)(r / (uint32_t)dimx);
    f3 dd;
    if (VOX && type == PT_VOXEL) {
        const u4 u = philox(r, p, 1u, 0u, seed, pass);
        const float w = u01(philox(r, p, 2u, 0u, seed, pass).a);
        dd = voxel_dir(ti, pi, dimx, dimy, u01(u.a), u01(u.b));
        *org = sample_point(g, type, u01(u.c), u01(u.d), w);
    } else {
        const u4 u = philox(r, p, (uint32_t)face, 0u, seed, pass);
        dd = diffuse_dir(xyz(g[3]), ti, pi, dimx, dimy, u01(u.a), u01(u.b));
        *org = sample_point(g, type, u01(u.c), u01(u.d), 0.f);
    }
    *dir = (face == 0) ? mk(-dd.x, -dd.y, -dd.z) : dd;
}

// ------------------------------------------------------------------ direct --
__device__ __forceinline__ bool direct_ray(const SourceDev &src, f3 org, f3 nrm, bool vox, uint32_t rx, uint32_t ry,
                                           double inv_nr, f3 *dir, float *tmax, double *strength) {
    if (src.type == 0) {
        f3 dd = normalize(mk(src.pos[0], src.pos[1], src.pos[2]));
        *dir = dd;
        *tmax = 1e38f;
        *strength = inv_nr * proj(nrm, dd, vox);
        return true;
    }
    f3 spos = mk(src.pos[0], src.pos[1], src.pos[2]);
    if (src.type == 1 || src.type == 2) {
        float ct = 1.0f - 2.0f * u01(rx);
        float st = sqrtf(fmaxf(0.f, 1.0f - ct * ct));
        float cp, sp;
        sincos2pi(u01(ry), &cp, &sp);
        float r = 0.5f * src.w0;
        f3 pt = mk(r * st * cp, r * st * sp, r * ct);
        f3 dd = sub(add(pt, spos), org);
        float dist = sqrtf(dot(dd, dd));
        dd = normalize(dd);
        double acc = 0.0;
        const int N = 10;
        for (int j = 0; j < N; ++j) {
            float cpj, spj;
            sincos2pi(((float)j + 0.5f) / (float)N, &cpj, &spj);
            for (int i = 0; i < N; ++i) {
                float cti = 1.0f - 2.0f * ((float)i + 0.5f) / (float)N;
                float sti = sqrtf(fmaxf(0.f, 1.0f - cti * cti));
                f3 l = mk(sti * cpj, sti * spj, cti);
                if (dot(l, dd) < 0.f) {
                    acc += inv_nr * proj(nrm, dd, vox) * (double)fabsf(dot(l, dd)) /
                           ((double)dist * (double)dist) / (double)(N * N) * (double)src.w0 * (double)src.w0;
                }
            }
        }
        *dir = dd;
        *tmax = dist;
        *strength = acc;
        return true;
    }
    if (src.type == 3 || src.type == 4) {
        f3 pt;
        if (src.type == 3) {
            pt = mk(src.w0 * (-0.5f + u01(rx)), src.w1 * (-0.5f + u01(ry)), 0.f);
        } else {
            float sx = -1.0f + 2.0f * u01(rx), sy = -1.0f + 2.0f * u01(ry);
            float r, ph;
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
            pt = mk(src.w0 * r * c, src.w0 * r * s, 0.f);
        }
        const float *R = src.R;
        f3 q = mk((R[0] * pt.x + R[1] * pt.y) + R[2] * pt.z, (R[3] * pt.x + R[4] * pt.y) + R[5] * pt.z,
                  (R[6] * pt.x + R[7] * pt.y) + R[8] * pt.z);
        f3 ldir = mk(R[2], R[5], R[8]);
        f3 dd = sub(add(q, spos), org);
        if (dot(dd, ldir) > 0.f) return false;
        float dist = sqrtf(dot(dd, dd));
        dd = normalize(dd);
        double area = (src.type == 3) ? (double)src.w0 * (double)src.w1 / 3.14159265358979323846
                                      : (double)src.w0 * (double)src.w0;
        *strength = inv_nr * proj(nrm, dd, vox) * (double)fabsf(dot(ldir, dd)) /
                    ((double)dist * (double)dist) * area;
        *dir = dd;
        *tmax = dist;
        return true;
    }
    return false;
}

template <bool STATS>
__global__ void __launch_bounds__(kBlock) k_direct(const DirectParams P) {
    const uint32_t R = (uint32_t)(P.dimx * P.dimy);
    const uint32_t total = P.count * R;
    const uint32_t stride = gridDim.x * blockDim.x;
    const double inv_nr = 1.0 / (double)R;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total; base += stride) {
        const uint32_t id = base + (threadIdx.x & 31);
        const bool active = id < total;
        const uint32_t p = active ? P.offset + id / R : 0u;
        const uint32_t r = active ? id % R : 0u;
        float4 g[4];
        int ts = 0;
        uint32_t type = 0;
        if (active) {
            load_rgen(P.sc, p, g);
            ts = P.sc.twosided[p];
            type = __float_as_uint(g[0].w);
        }
        for (int k = 0; k < P.S; ++k) {
            uint32_t nv = 0, np = 0;
            double v[2] = {0.0, 0.0};  // [face0, face1]
            bool live = active;
            if (live) {
                const uint32_t c2 = (uint32_t)(k << 1);
                u4 u = philox(r, p, c2, 0u, P.seed, P.pass);
                const bool vox = type == PT_VOXEL;
                f3 org = direct_origin(g, type, r, p, c2, P.dimx, P.dimy, P.seed, P.pass, u);
                f3 nrm = xyz(g[3]);
                f3 dir;
                float tmax;
                double strength;
                live = direct_ray(P.src[k], org, nrm, vox, u.c, u.d, inv_nr, &dir, &tmax, &strength);
                if (live) {
                    bool face = vox || dot(dir, nrm) > 0.f;
                    if ((!face && ts == 0) || ts == 3) {
                        live = false;
                    } else {
                        Hit h = trace_full<STATS>(P.sc, org, dir, 1e-4f, tmax, true, VoxKey{r, p, c2, P.seed, P.pass},
                                                  &nv, &np);
                        if (h.prim == 0xFFFFFFFFu) v[face ? 1 : 0] = strength;
                    }
                }
            }
            count_rays(P.sc, live);
            if (STATS) count_visits(P.sc, nv, np);
            // sums land at G[(p*S + k)*2 + face]
            uint32_t key = active ? (p * (uint32_t)P.S + (uint32_t)k) : 0xFFFFFFFFu;
            warp_segment_add<2>(key, v, 2, P.G, 2);
        }
    }
}

// ------------------------------------------------------------------ diffuse --
__device__ __forceinline__ double sky_fd(f3 dir, const SkyParams &sky, int b) {
    float K = sky.K ? sky.K[b] : 0.f;
    if (K > 0.f) {
        f3 pk = mk(sky.peak[3 * b], sky.peak[3 * b + 1], sky.peak[3 * b + 2]);
        double c = fmax(-1.0, fmin(1.0, (double)dot(pk, dir)));
        double psi = fmax(acos(c), 3.14159265358979323846 / 180.0);
        return pow(psi, -(double)K) * (double)(sky.knorm ? sky.knorm[b] : 1.f);
    }
    if (sky.prague && sky.prague[4 * b + 3] > 0.f) {
        f3 pk = sky.peak ? mk(sky.peak[3 * b], sky.peak[3 * b + 1], sky.peak[3 * b + 2]) : mk(0.f, 0.f, 1.f);
        const float *pr = sky.prague + 4 * b;
        double c = fmax(-1.0, fmin(1.0, (double)dot(dir, pk)));
        double gamma = acos(c) * 180.0 / 3.14159265358979323846;
        double cth = fmax((double)dir.z, 0.0);
        double pat = (1.0 + pr[0] * exp(-gamma / pr[1])) * (1.0 + (pr[2] - 1.0) * (1.0 - cth));
        return pat * pr[3] * 3.14159265358979323846;
    }
    return 1.0;
}

template <int NB, bool STATS>
__global__ void __launch_bounds__(kBlock) k_diffuse(const DiffuseParams P) {
    const uint32_t R = (uint32_t)(P.dimx * P.dimy);
    const uint32_t total = P.count * R;
    const uint32_t stride = gridDim.x * blockDim.x;
    // blockIdx.y: 0 = top face (launch_face 1), 1 = bottom face (launch_face 0)
    const int face = (blockIdx.y == 0) ? 1 : 0;
    if (!(P.faces & (1 << blockIdx.y))) return;
    double *G = face ? P.Gt : P.Gb;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total; base += stride) {
        const uint32_t id = base + (threadIdx.x & 31);
        bool active = id < total;
        const uint32_t p = active ? P.offset + id / R : 0u;
        const uint32_t r = active ? id % R : 0u;
        if (active) {
            int ts = P.sc.twosided[p];
            if (face == 1 && ts == 3) active = false;
            if (face == 0 && ts != 1) active = false;
        }
        double v[NB];
#pragma unroll
        for (int j = 0; j < NB; ++j) v[j] = 0.0;
        uint32_t nv = 0, np = 0;
        if (active) {
            float4 g[4];
            load_rgen(P.sc, p, g);
            uint32_t type = __float_as_uint(g[0].w);
            f3 org, dir;
            diffuse_ray<true>(g, type, r, p, face, P.dimx, P.dimy, P.seed, P.pass, &org, &dir);
            Hit h = trace_full<STATS>(P.sc, org, dir, 1e-4f, 1e38f, false, VoxKey{r, p, (uint32_t)face, P.seed, P.pass},
                                      &nv, &np);
            if (h.prim == kLost) {
                // dropped ray: no deposit
            } else if (h.prim != 0xFFFFFFFFu) {
                const float *src = (h.face ? P.otop : P.obot) + (size_t)h.prim * P.Bl;
#pragma unroll
                for (int j = 0; j < NB; ++j)
                    if (j < P.Bc) v[j] = (double)__ldg(src + j);
            } else {
#pragma unroll
                for (int j = 0; j < NB; ++j)
                    if (j < P.Bc) {
                        float fl = P.sky.flux[j];
                        if (fl > 0.f) v[j] = sky_fd(dir, P.sky, j) * (double)fl;
                    }
            }
        }
        count_rays(P.sc, active);
        if (STATS) count_visits(P.sc, nv, np);
        uint32_t key = active ? p : 0xFFFFFFFFu;
        warp_segment_add<NB>(key, v, P.Bc, G, P.Bl);
    }
}

// ------------------------------------------------------- persistent diffuse --
// Persistent threads with dynamic ray fetch and speculative while-while traversal
// (after Aila & Laine, "Understanding the Efficiency of Ray Traversal on GPUs",
// HPG 2009): a lane whose ray has ended takes the next ray id from a global
// counter at the top of the next round, so lanes do not idle until the longest
// ray of the warp ends; leaves are postponed until every active lane has one, so
// node visits and primitive tests run in separate, convergent loops.  Hit results
// equal those of trace_bvh (same tests, same tie rule; only the order differs).
// Each lane keeps a running FP64 sum for its current origin (primitive, face) and
// adds it to G only when the origin changes.
constexpr int32_t kSentinel = 0x7FFFFFF0;

// MINB: resident blocks per SM the register allocation must allow (4, the default: 64
// registers; 3: more registers, fewer warps).  VOX: the scene holds voxels (turbid media
// with their own ray sampling); without it the voxel code is left out.
template <int NB, bool RECORD, int MINB, bool VOX>
__global__ void __launch_bounds__(kBlock, MINB) k_diffuse_ps(const DiffuseParams P) {
    unsigned long long *fetch = P.fetch;
    const int lane = threadIdx.x & 31;
    const uint32_t R = (uint32_t)(P.dimx * P.dimy);
    const uint32_t per_face = P.count * R;
    const int nf = ((P.faces & 1) ? 1 : 0) + ((P.faces & 2) ? 1 : 0);
    const unsigned long long total = (unsigned long long)per_face * (unsigned long long)nf;
    const uint32_t ni = (uint32_t)(P.sc.n > 1 ? P.sc.n - 1 : 1);
    const TraceScene &sc = P.sc;

    bool live = false, exhausted = false;
    f3 o = mk(0.f, 0.f, 0.f), d = o, inv = o, ooi = o;
    WT w = wt_setup(mk(0.f, 0.f, 1.f));
    float best = 1e38f;
    uint32_t bprim = 0xFFFFFFFFu;
    int bface = 0;
    int32_t cur = kSentinel, leaf = 0;
    int sp = 0;
    int32_t stack[kStack];
    uint32_t budget = 0;
    int wraps = 0;
    uint32_t p = 0, rr = 0;
    int face = 1;
    unsigned long long rid = 0;
    uint32_t akey = 0xFFFFFFFFu;
    // running sums live in shared memory (one slot row per thread) to keep registers
    // for the traversal state
    __shared__ double s_sum[NB][kBlock];
    double *sum_j = &s_sum[0][threadIdx.x];
#define ACC(j) sum_j[(j) * kBlock]
#pragma unroll
    for (int j = 0; j < NB; ++j) ACC(j) = 0.0;
    unsigned long long nrays = 0;

    for (;;) {
        // ---- refill lanes without a ray
        const bool need = !live && !exhausted;
        const unsigned m = __ballot_sync(0xffffffffu, need);
        if (m) {
            const int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(fetch, (unsigned long long)__popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need) {
                const unsigned long long id = base + (unsigned long long)__popc(m & ((1u << lane) - 1u));
                if (id >= total) {
                    exhausted = true;
                } else {
                    rid = id;
                    const uint32_t fi = (uint32_t)(id / per_face);
                    const uint32_t rem = (uint32_t)(id - (unsigned long long)fi * per_face);
                    face = (nf == 2) ? (fi == 0 ? 1 : 0) : ((P.faces & 1) ? 1 : 0);
                    p = P.offset + rem / R;
                    const uint32_t r = rem % R;
                    const int ts = sc.twosided[p];
                    const bool skip = (face == 1 && ts == 3) || (face == 0 && ts != 1);
                    if (!skip) {
                        float4 g[4];
                        load_rgen(sc, p, g);
                        const uint32_t type = __float_as_uint(g[0].w);
                        diffuse_ray<VOX>(g, type, r, p, face, P.dimx, P.dimy, P.seed, P.pass, &o, &d);
                        if (VOX) rr = r;
                        w = wt_setup(d);
                        inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
                        ooi = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
                        best = 1e38f;
                        bprim = 0xFFFFFFFFu;
                        bface = 0;
                        cur = (sc.n > 0) ? 0 : kSentinel;
                        leaf = 0;
                        sp = 0;
                        budget = 2u * (uint32_t)sc.n + 64u;
                        wraps = 0;
                        live = true;
                        ++nrays;
                    }
                }
            }
        }
        // A lane may be idle because its id was skipped by the face rule; only when every
        // lane has run past the end of the id range is the warp done.
        if (__all_sync(0xffffffffu, exhausted && !live)) break;
        if (!live) continue;

        // ---- internal nodes; leaves are postponed
        while (cur >= 0 && cur != kSentinel) {
            if ((uint32_t)cur >= ni || budget-- == 0u) {
                raise(sc.status, ERR_BOUNDS);
                cur = kSentinel;
                leaf = 0;
                break;
            }
            const float4 *nd = sc.nodes + 4 * (size_t)cur;
            const float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3);
            int32_t c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
            float tn0, tn1;
            const bool h0 = c0 != kEmptyChild &&
                            slab_node(ooi, inv, mk(n0.x, n0.y, n0.z), mk(n0.w, n1.x, n1.y), 1e-4f, best, &tn0);
            const bool h1 = c1 != kEmptyChild &&
                            slab_node(ooi, inv, mk(n1.z, n1.w, n2.x), mk(n2.y, n2.z, n2.w), 1e-4f, best, &tn1);
            if (!h0 && !h1) {
                cur = sp > 0 ? stack[--sp] : kSentinel;
            } else {
                cur = h0 ? c0 : c1;
                if (h0 && h1) {
                    int32_t farc = c1;
                    if (tn1 < tn0) {
                        cur = c1;
                        farc = c0;
                    }
                    if (sp >= kStack) {
                        raise(sc.status, ERR_STACK);
                        cur = kSentinel;
                        leaf = 0;
                        break;
                    }
                    stack[sp++] = farc;
                }
            }
            if (cur < 0 && leaf == 0) {
                leaf = cur;
                cur = sp > 0 ? stack[--sp] : kSentinel;
            }
            if (__all_sync(__activemask(), leaf != 0)) break;
        }
        // ---- primitive tests
        while (leaf != 0) {
            const uint32_t slot = (uint32_t)(~leaf);
            if (slot < (uint32_t)sc.n) {
                float t;
                int fc;
                uint32_t orig;
                const VoxKey vk{rr, p, (uint32_t)face | ((uint32_t)wraps << 16), P.seed, P.pass};
                if (rec_hit<VOX>(sc.rec, slot, w, o, d, inv, 1e-4f, best, vk, &t, &fc, &orig)) {
                    if (bprim == 0xFFFFFFFFu || t < best || (t == best && orig < bprim)) {
                        best = t;
                        bprim = orig;
                        bface = fc;
                    }
                }
            } else {
                raise(sc.status, ERR_BOUNDS);
            }
            leaf = 0;
            if (cur < 0) {
                leaf = cur;
                cur = sp > 0 ? stack[--sp] : kSentinel;
            }
        }
        if (cur != kSentinel || leaf != 0) continue;  // traversal of this ray goes on next round

        // ---- periodic walls: wrap and restart, or finish the ray
        bool lost = false;
        if (sc.nbbox > 0) {
            float tb;
            int which = -1;
            if (wall_closest(sc, o, d, 1e-4f, (bprim != 0xFFFFFFFFu) ? best : 1e38f, &tb, &which) &&
                (bprim == 0xFFFFFFFFu || tb < best)) {
                if (wraps >= 9) {
                    lost = true;
                } else {
                    f3 hp = add(o, scl(d, tb));
                    if ((sc.periodic_x == 1.f) && which < 2) {
                        float width = sc.bbox[4].x - sc.bbox[0].x;
                        hp.x = hp.x + ((which == 0) ? width : -width);
                    } else {
                        int yb = (sc.periodic_x == 1.f) ? 2 : 0;
                        float width = sc.bbox[4 * (yb + 1)].y - sc.bbox[4 * yb].y;
                        hp.y = hp.y + ((which == yb) ? width : -width);
                    }
                    o = hp;
                    ooi = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
                    best = 1e38f;
                    bprim = 0xFFFFFFFFu;
                    cur = 0;
                    sp = 0;
                    budget = 2u * (uint32_t)sc.n + 64u;
                    ++wraps;
                    continue;
                }
            }
        }
        // ---- value of the finished ray, added to the lane's running sum
        live = false;
        if (RECORD) {
            P.hits[rid] = lost ? kLostCode : ((bprim == 0xFFFFFFFFu) ? kMissCode : ((bprim << 1) | (uint32_t)bface));
            continue;
        }
        if (lost) continue;
        const uint32_t key = 2u * p + (uint32_t)face;
        if (key != akey) {
            if (akey != 0xFFFFFFFFu) {
                double *dst = ((akey & 1u) ? P.Gt : P.Gb) + (size_t)(akey >> 1) * P.Bl;
#pragma unroll
                for (int j = 0; j < NB; ++j)
                    if (j < P.Bc && ACC(j) != 0.0) atomicAdd(dst + j, ACC(j));
            }
            akey = key;
#pragma unroll
            for (int j = 0; j < NB; ++j) ACC(j) = 0.0;
        }
        if (bprim != 0xFFFFFFFFu) {
            const float *src = (bface ? P.otop : P.obot) + (size_t)bprim * P.Bl;
#pragma unroll
            for (int j = 0; j < NB; ++j)
                if (j < P.Bc) ACC(j) += (double)__ldg(src + j);
        } else {
#pragma unroll
            for (int j = 0; j < NB; ++j)
                if (j < P.Bc) {
                    float fl = P.sky.flux[j];
                    if (fl > 0.f) ACC(j) += sky_fd(d, P.sky, j) * (double)fl;
                }
        }
    }
    if (akey != 0xFFFFFFFFu) {
        double *dst = ((akey & 1u) ? P.Gt : P.Gb) + (size_t)(akey >> 1) * P.Bl;
#pragma unroll
        for (int j = 0; j < NB; ++j)
            if (j < P.Bc && ACC(j) != 0.0) atomicAdd(dst + j, ACC(j));
    }
    if (sc.rays && nrays) atomicAdd(sc.rays, nrays);
#undef ACC
}

// ------------------------------------------------------------------ testing --
__global__ void k_trace_rays(const TraceScene sc, int64_t nrays, const float *__restrict__ o,
                             const float *__restrict__ d, float tmin, float tmax, int anyhit, int32_t *hit, float *t,
                             int32_t *face) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrays) return;
    f3 oo = mk(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
    f3 dd = mk(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
    uint32_t nv = 0, np = 0;
    // voxel draws of explicit ray i: counter (i, i >> 32, 2^31), key (0, ~0)
    const VoxKey vk{(uint32_t)i, (uint32_t)((uint64_t)i >> 32), 0x80000000u, 0u, 0xFFFFFFFFu};
    Hit h = trace_bvh<false>(sc, oo, dd, tmin, tmax, anyhit != 0, vk, &nv, &np);
    hit[i] = (h.prim == 0xFFFFFFFFu) ? -1 : (int32_t)h.prim;
    t[i] = h.t;
    face[i] = h.face;
}

__global__ void k_gen_rays(const TraceScene sc, int kind, uint32_t seed, uint32_t pass, int dimx, int dimy, int face,
                           float dx, float dy, float dz, float *o, float *d) {
    const uint32_t R = (uint32_t)(dimx * dimy);
    const int64_t total = (int64_t)sc.n * R;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    uint32_t p = (uint32_t)(i / R), r = (uint32_t)(i % R);
    float4 g[4];
    load_rgen(sc, p, g);
    uint32_t type = __float_as_uint(g[0].w);
    f3 org, dir;
    if (kind == 0) {
        const u4 u = philox(r, p, (uint32_t)face, 0u, seed, pass);
        org = direct_origin(g, type, r, p, (uint32_t)face, dimx, dimy, seed, pass, u);
        dir = normalize(mk(dx, dy, dz));
    } else {
        diffuse_ray<true>(g, type, r, p, face, dimx, dimy, seed, pass, &org, &dir);
    }
    o[3 * i] = org.x;
    o[3 * i + 1] = org.y;
    o[3 * i + 2] = org.z;
    d[3 * i] = dir.x;
    d[3 * i + 1] = dir.y;
    d[3 * i + 2] = dir.z;
}

// ------------------------------------------------------------------ epilogues --
// compacted band b -> global band of the b-th set flag
__device__ __forceinline__ int global_band(const uint8_t *flags, int Bg, int b) {
    int c = -1;
    for (int bg = 0; bg < Bg; ++bg) {
        if (!flags[bg]) continue;
        if (++c == b) return bg;
    }
    return -1;
}

__global__ void k_epilogue_diffuse(const EpilogueParams P) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)P.n * P.Bc) return;
    int p = (int)(i / P.Bc), b = (int)(i % P.Bc);
    int bg = global_band(P.flags, P.Bg, b);
    size_t k = (size_t)p * P.Bl + b;
    double gt = P.Gt[k] * P.strength, gb = P.Gb[k] * P.strength;
    size_t m = (size_t)p * P.Bg + bg;  // source 0
    double rho = P.rho[m], tau = P.tau[m];
    P.rin[k] += (gt + gb) * (1.0 - rho - tau);
    if (rho > 0.0 || tau > 0.0) {
        P.stop[k] += gt * rho + gb * tau;
        P.sbot[k] += gt * tau + gb * rho;
    }
}

__global__ void k_epilogue_direct(const EpilogueParams P) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)P.n * P.Bc) return;
    int p = (int)(i / P.Bc), b = (int)(i % P.Bc);
    int bg = global_band(P.flags, P.Bg, b);
    size_t k = (size_t)p * P.Bl + b;
    double in = 0.0, top = 0.0, bot = 0.0;
    for (int s = 0; s < P.S; ++s) {
        double flux = (double)P.src_flux[(size_t)s * P.Bl + b];
        double g0 = P.Gd[((size_t)p * P.S + s) * 2] * flux, g1 = P.Gd[((size_t)p * P.S + s) * 2 + 1] * flux;
        size_t m = ((size_t)s * P.n + p) * P.Bg + bg;
        double rho = P.rho[m], tau = P.tau[m];
        in += (g0 + g1) * (1.0 - rho - tau);
        if (rho > 0.0 || tau > 0.0) {
            top += g1 * rho + g0 * tau;
            bot += g1 * tau + g0 * rho;
        }
    }
    P.rin[k] += in;
    P.stop[k] += top;
    P.sbot[k] += bot;
}

__global__ void k_to_float(const double *__restrict__ a, float *__restrict__ out, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)a[i];
}

__global__ void k_fold(int n, int Bl, const int8_t *__restrict__ ts, const double *__restrict__ stop,
                       const double *__restrict__ sbot, double *__restrict__ ftop, double *__restrict__ fbot) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n * Bl) return;
    int p = (int)(i / Bl);
    double a = stop[i], b = sbot[i];
    if (ts[p] == 0) {
        double t = a + b;
        ftop[i] = t;
        fbot[i] = t;
    } else {
        ftop[i] = a;
        fbot[i] = b;
    }
}

__global__ void k_emission(int n, int Bl, const uint8_t *__restrict__ em, const int32_t *__restrict__ depth,
                           const float *__restrict__ eps, const float *__restrict__ temp, const int8_t *__restrict__ ts,
                           double *__restrict__ ftop, double *__restrict__ fbot) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n * Bl) return;
    int p = (int)(i / Bl), b = (int)(i % Bl);
    if (!em[b]) return;
    const float sigma = 5.6703744e-8f;
    float e = eps[i];
    if (depth[b] == 0 && e != 1.f) e = 1.f;
    double T = (double)temp[p];
    float out = (float)((double)(sigma * e) * (T * T * T * T));
    ftop[i] += out;
    if (ts[p] != 0) fbot[i] += out;
}

__global__ void k_final(size_t nb, const double *__restrict__ rin, const double *__restrict__ stop,
                        const double *__restrict__ sbot, float *__restrict__ out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nb) out[i] = (float)((rin[i] + stop[i]) + sbot[i]);
}


// ---------------------------------------------------------------- batched sweep --
// Shadow rays of many suns in one launch.  Ray ids are sun-major, so a warp holds
// 32 strata of one primitive toward ONE sun (coherent rays).  Origins and strengths
// are exactly those of a plain direct pass with the same seed (source slot 0).
__global__ void __launch_bounds__(kBlock) k_direct_sweep(const SweepDirectParams P) {
    const uint32_t R = (uint32_t)(P.dimx * P.dimy);
    const unsigned long long per_sun = (unsigned long long)P.sc.n * R;
    const unsigned long long total = per_sun * (unsigned long long)P.nsun;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const double inv_nr = 1.0 / (double)R;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total;
         base += stride) {
        const unsigned long long id = base + (threadIdx.x & 31);
        const bool active = id < total;
        uint32_t sun = 0, p = 0, r = 0;
        if (active) {
            sun = (uint32_t)(id / per_sun);
            const unsigned long long rem = id - (unsigned long long)sun * per_sun;
            p = (uint32_t)(rem / R);
            r = (uint32_t)(rem % R);
        }
        double v[2] = {0.0, 0.0};
        bool live = false;
        if (active) {
            float4 g[4];
            load_rgen(P.sc, p, g);
            const int ts = P.sc.twosided[p];
            const uint32_t type = __float_as_uint(g[0].w);
            const u4 u = philox(r, p, 0u, 0u, P.seed, 0u);
            const f3 org = direct_origin(g, type, r, p, 0u, P.dimx, P.dimy, P.seed, 0u, u);
            const f3 nrm = xyz(g[3]);
            const f3 dd = normalize(mk(P.sun_dir[3 * sun], P.sun_dir[3 * sun + 1], P.sun_dir[3 * sun + 2]));
            const double strength = inv_nr * (double)fabsf(dot(nrm, dd));
            const bool face = dot(dd, nrm) > 0.f;
            if (!((!face && ts == 0) || ts == 3)) {
                live = true;
                uint32_t nv = 0, np = 0;
                const Hit h = trace_full<false>(P.sc, org, dd, 1e-4f, 1e38f, true, VoxKey{r, p, 0u, P.seed, 0u}, &nv, &np);
                if (h.prim == 0xFFFFFFFFu) v[face ? 1 : 0] = strength;
            }
        }
        count_rays(P.sc, live);
        const uint32_t key = active ? (p * (uint32_t)P.nsun + sun) : 0xFFFFFFFFu;
        warp_segment_add<2>(key, v, 2, P.G, 2);
    }
}

// One warp per (face, primitive): lanes run over channels, the R recorded hits of the
// primitive are read in order, so every sum is deterministic.  A hit reads the row
// radiation_out[hit][0..C) (coalesced); a miss adds the channel's sky flux.
template <int CPL>
__global__ void __launch_bounds__(256) k_gather(const GatherParams P) {
    const int lane = threadIdx.x & 31;
    const int nf = ((P.faces & 1) ? 1 : 0) + ((P.faces & 2) ? 1 : 0);
    const long long items = (long long)nf * P.n;
    const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long item = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; item < items; item += warps) {
        const int fi = (int)(item / P.n);
        const int p = (int)(item % P.n);
        const int face = (nf == 2) ? (fi == 0 ? 1 : 0) : ((P.faces & 1) ? 1 : 0);
        const int ts = P.twosided[p];
        if ((face == 1 && ts == 3) || (face == 0 && ts != 1)) {  // face not launched: its sums are zero
            double *G = (face ? P.Gt : P.Gb) + (size_t)p * P.C;
            for (int c = lane; c < P.C; c += 32) G[c] = 0.0;
            continue;
        }
        double acc[CPL];
#pragma unroll
        for (int k = 0; k < CPL; ++k) acc[k] = 0.0;
        const uint32_t *row = P.hits + ((size_t)fi * P.n + p) * P.R;
        for (int r = 0; r < P.R; ++r) {
            const uint32_t h = __ldg(row + r);
            if (h == kLostCode) continue;
            if (h == kMissCode) {
#pragma unroll
                for (int k = 0; k < CPL; ++k) {
                    const int c = lane + 32 * k;
                    if (c < P.C) acc[k] += (double)__ldg(P.sky + c);
                }
            } else {
                const float *src = ((h & 1u) ? P.otop : P.obot) + (size_t)(h >> 1) * P.C;
#pragma unroll
                for (int k = 0; k < CPL; ++k) {
                    const int c = lane + 32 * k;
                    if (c < P.C) acc[k] += (double)__ldg(src + c);
                }
            }
        }
        double *G = (face ? P.Gt : P.Gb) + (size_t)p * P.C;
#pragma unroll
        for (int k = 0; k < CPL; ++k) {
            const int c = lane + 32 * k;
            if (c < P.C) G[c] = acc[k];
        }
    }
}

__global__ void k_epilogue_diffuse_channels(const ChannelEpilogue P) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)P.n * P.C) return;
    const int p = (int)(i / P.C), c = (int)(i % P.C), b = c % P.Bl;
    if (!P.mask[c]) return;
    const double gt = P.Gt[i] * P.strength, gb = P.Gb[i] * P.strength;
    const double rho = P.rho[(size_t)p * P.Bl + b], tau = P.tau[(size_t)p * P.Bl + b];
    P.rin[i] += (gt + gb) * (1.0 - rho - tau);
    if (rho > 0.0 || tau > 0.0) {
        P.stop[i] += gt * rho + gb * tau;
        P.sbot[i] += gt * tau + gb * rho;
    }
}

__global__ void k_epilogue_direct_channels(const ChannelEpilogue P, int nsun) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)P.n * P.C) return;
    const int p = (int)(i / P.C), c = (int)(i % P.C), b = c % P.Bl, sun = c / P.Bl;
    if (!P.mask[c]) return;
    const double flux = (double)P.flux[c];
    const double g0 = P.Gd[((size_t)p * nsun + sun) * 2] * flux, g1 = P.Gd[((size_t)p * nsun + sun) * 2 + 1] * flux;
    const double rho = P.rho[(size_t)p * P.Bl + b], tau = P.tau[(size_t)p * P.Bl + b];
    P.rin[i] += (g0 + g1) * (1.0 - rho - tau);
    if (rho > 0.0 || tau > 0.0) {
        P.stop[i] += g1 * rho + g0 * tau;
        P.sbot[i] += g1 * tau + g0 * rho;
    }
}

__global__ void k_copy_channels(int n, int C, const uint8_t *__restrict__ mask, double *st, double *sb, float *ot,
                                float *ob, int zero) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)n * C) return;
    if (!mask[i % C]) return;
    ot[i] = (float)st[i];
    ob[i] = (float)sb[i];
    if (zero) {
        st[i] = 0.0;
        sb[i] = 0.0;
    }
}

__global__ void k_fold_channels(int n, int C, const uint8_t *__restrict__ mask, const int8_t *__restrict__ ts,
                                double *st, double *sb, float *ot, float *ob) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)n * C) return;
    const int p = (int)(i / C);
    if (!mask[i % C]) {
        ot[i] = 0.f;
        ob[i] = 0.f;
        return;
    }
    const double a = st[i], b = sb[i];
    if (ts[p] == 0) {
        const double t = a + b;
        ot[i] = (float)t;
        ob[i] = (float)t;
    } else {
        ot[i] = (float)a;
        ob[i] = (float)b;
    }
    st[i] = 0.0;
    sb[i] = 0.0;
}


inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

template <bool STATS>
static cudaError_t direct_impl(const DirectParams &p, int max_blocks, cudaStream_t s) {
    int64_t total = (int64_t)p.count * p.dimx * p.dimy;
    if (total <= 0 || p.S <= 0) return cudaSuccess;
    unsigned nb = blocks_for(total, kBlock);
    if ((int)nb > max_blocks) nb = (unsigned)max_blocks;
    k_direct<STATS><<<nb, kBlock, 0, s>>>(p);
    return cudaGetLastError();
}

static int ps_min_blocks() {
    static int v = -1;
    if (v < 0) {
        const char *e = getenv("HRT_PS_MINB");
        v = (e && e[0] == '3') ? 3 : 4;
    }
    return v;
}

template <int NB, int MINB, bool VOX>
static cudaError_t diffuse_ps_launch_b(const DiffuseParams &p, cudaStream_t s) {
    static int blocks_per_sm = 0, sms = 0;
    if (blocks_per_sm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_diffuse_ps<NB, false, MINB, VOX>, kBlock, 0);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    cudaError_t e = cudaMemsetAsync(p.fetch, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    k_diffuse_ps<NB, false, MINB, VOX><<<sms * blocks_per_sm, kBlock, 0, s>>>(p);
    return cudaGetLastError();
}

// minb: 4 or 3 (resident blocks per SM the register budget allows); 0 = the default.
template <int NB>
static cudaError_t diffuse_ps_launch(const DiffuseParams &p, int minb, cudaStream_t s) {
    if (p.sc.voxels) return diffuse_ps_launch_b<NB, 4, true>(p, s);
    if (minb == 0) minb = ps_min_blocks();
    return minb == 4 ? diffuse_ps_launch_b<NB, 4, false>(p, s) : diffuse_ps_launch_b<NB, 3, false>(p, s);
}

static bool use_persistent() {
    static int v = -1;
    if (v < 0) {
        const char *e = getenv("HRT_TRAVERSAL");
        v = (e && e[0] == 's') ? 0 : 1;  // "simple" selects the one-ray-per-thread kernel
    }
    return v == 1;
}

// variant: DV_DEFAULT (persistent unless HRT_TRAVERSAL=simple), DV_PS4 / DV_PS3 (persistent,
// 4 or 3 resident blocks per SM), DV_SIMPLE (one ray per thread).
template <bool STATS>
static cudaError_t diffuse_impl(const DiffuseParams &p, int variant, int max_blocks, cudaStream_t s) {
    int64_t total = (int64_t)p.count * p.dimx * p.dimy;
    if (total <= 0 || p.Bc <= 0) return cudaSuccess;
    const bool persistent = variant == DV_DEFAULT ? use_persistent() : variant != DV_SIMPLE;
    if (!STATS && p.fetch && persistent) {
        const int minb = variant == DV_PS4 ? 4 : (variant == DV_PS3 ? 3 : 0);
        if (p.Bc <= 1) return diffuse_ps_launch<1>(p, minb, s);
        if (p.Bc <= 2) return diffuse_ps_launch<2>(p, minb, s);
        if (p.Bc <= 4) return diffuse_ps_launch<4>(p, minb, s);
        if (p.Bc <= 8) return diffuse_ps_launch<8>(p, minb, s);
        if (p.Bc <= 16) return diffuse_ps_launch<16>(p, minb, s);
        return cudaErrorInvalidValue;
    }
    unsigned nb = blocks_for(total, kBlock);
    if ((int)nb > max_blocks) nb = (unsigned)max_blocks;
    dim3 grid(nb, 2);
    if (p.Bc <= 1) k_diffuse<1, STATS><<<grid, kBlock, 0, s>>>(p);
    else if (p.Bc <= 2) k_diffuse<2, STATS><<<grid, kBlock, 0, s>>>(p);
    else if (p.Bc <= 4) k_diffuse<4, STATS><<<grid, kBlock, 0, s>>>(p);
    else if (p.Bc <= 8) k_diffuse<8, STATS><<<grid, kBlock, 0, s>>>(p);
    else if (p.Bc <= 16) k_diffuse<16, STATS><<<grid, kBlock, 0, s>>>(p);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_direct(const DirectParams &p, int max_blocks, cudaStream_t s) {
    return direct_impl<false>(p, max_blocks, s);
}
cudaError_t launch_diffuse(const DiffuseParams &p, int max_blocks, cudaStream_t s) {
    return diffuse_impl<false>(p, DV_DEFAULT, max_blocks, s);
}
cudaError_t launch_diffuse_variant(const DiffuseParams &p, int variant, int max_blocks, cudaStream_t s) {
    return diffuse_impl<false>(p, variant, max_blocks, s);
}
cudaError_t launch_direct_stats(const DirectParams &p, int max_blocks, cudaStream_t s) {
    return direct_impl<true>(p, max_blocks, s);
}
cudaError_t launch_diffuse_stats(const DiffuseParams &p, int max_blocks, cudaStream_t s) {
    return diffuse_impl<true>(p, DV_DEFAULT, max_blocks, s);
}

cudaError_t launch_trace_rays(const TraceScene &sc, int64_t nrays, const float *o, const float *d, float tmin,
                              float tmax, int anyhit, int32_t *hit, float *t, int32_t *face, cudaStream_t s) {
    if (nrays <= 0) return cudaSuccess;
    k_trace_rays<<<blocks_for(nrays, 128), 128, 0, s>>>(sc, nrays, o, d, tmin, tmax, anyhit, hit, t, face);
    return cudaGetLastError();
}

cudaError_t launch_gen_rays(const TraceScene &sc, int kind, uint32_t seed, uint32_t pass, int dimx, int dimy,
                            int face, float dx, float dy, float dz, float *o, float *d, cudaStream_t s) {
    int64_t total = (int64_t)sc.n * dimx * dimy;
    if (total <= 0) return cudaSuccess;
    k_gen_rays<<<blocks_for(total, 128), 128, 0, s>>>(sc, kind, seed, pass, dimx, dimy, face, dx, dy, dz, o, d);
    return cudaGetLastError();
}

cudaError_t launch_epilogue_direct(const EpilogueParams &p, cudaStream_t s) {
    int64_t n = (int64_t)p.n * p.Bc;
    if (n <= 0) return cudaSuccess;
    k_epilogue_direct<<<blocks_for(n, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_epilogue_diffuse(const EpilogueParams &p, cudaStream_t s) {
    int64_t n = (int64_t)p.n * p.Bc;
    if (n <= 0) return cudaSuccess;
    k_epilogue_diffuse<<<blocks_for(n, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_to_float(const double *a, float *out, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_to_float<<<blocks_for((int64_t)n, 256), 256, 0, s>>>(a, out, n);
    return cudaGetLastError();
}

cudaError_t launch_fold_onesided(int n, int Bl, const int8_t *twosided, const double *stop, const double *sbot,
                                 double *ftop, double *fbot, cudaStream_t s) {
    int64_t m = (int64_t)n * Bl;
    if (m <= 0) return cudaSuccess;
    k_fold<<<blocks_for(m, 256), 256, 0, s>>>(n, Bl, twosided, stop, sbot, ftop, fbot);
    return cudaGetLastError();
}

cudaError_t launch_emission(int n, int Bl, const uint8_t *emission, const int32_t *depth, const float *eps,
                            const float *temperature, const int8_t *twosided, double *ftop, double *fbot,
                            cudaStream_t s) {
    int64_t m = (int64_t)n * Bl;
    if (m <= 0) return cudaSuccess;
    k_emission<<<blocks_for(m, 256), 256, 0, s>>>(n, Bl, emission, depth, eps, temperature, twosided, ftop, fbot);
    return cudaGetLastError();
}

cudaError_t launch_final_flux(size_t nb, const double *rin, const double *stop, const double *sbot, float *out,
                              cudaStream_t s) {
    if (nb == 0) return cudaSuccess;
    k_final<<<blocks_for((int64_t)nb, 256), 256, 0, s>>>(nb, rin, stop, sbot, out);
    return cudaGetLastError();
}

// Scattering residual per band: num = sum_p area_p (stop + sbot), den = sum_p area_p
// (rin + stop + sbot), in FP64 by a fixed two-stage reduction (grid-stride partial sums
// in a fixed order, a shared-memory tree per block, block partials added in block
// order), so the result does not depend on scheduling.
__global__ void __launch_bounds__(256) k_residual(int n, int Bl, const double *__restrict__ area,
                                                  const double *__restrict__ rin, const double *__restrict__ stop,
                                                  const double *__restrict__ sbot, double *__restrict__ partial) {
    __shared__ double sh[2][256];
    const int tid = threadIdx.x;
    for (int b = 0; b < Bl; ++b) {
        double num = 0.0, den = 0.0;
        for (int p = blockIdx.x * blockDim.x + tid; p < n; p += gridDim.x * blockDim.x) {
            const size_t i = (size_t)p * Bl + b;
            const double sc = stop[i] + sbot[i];
            num += area[p] * sc;
            den += area[p] * (rin[i] + sc);
        }
        sh[0][tid] = num;
        sh[1][tid] = den;
        __syncthreads();
        for (int off = 128; off > 0; off >>= 1) {
            if (tid < off) {
                sh[0][tid] += sh[0][tid + off];
                sh[1][tid] += sh[1][tid + off];
            }
            __syncthreads();
        }
        if (tid == 0) {
            partial[((size_t)blockIdx.x * Bl + b) * 2] = sh[0][0];
            partial[((size_t)blockIdx.x * Bl + b) * 2 + 1] = sh[1][0];
        }
        __syncthreads();
    }
}

__global__ void k_residual_final(int nblocks, int Bl, const double *__restrict__ partial, double *__restrict__ out) {
    const int b = threadIdx.x;
    if (b >= Bl) return;
    double num = 0.0, den = 0.0;
    for (int k = 0; k < nblocks; ++k) {
        num += partial[((size_t)k * Bl + b) * 2];
        den += partial[((size_t)k * Bl + b) * 2 + 1];
    }
    out[2 * b] = num;
    out[2 * b + 1] = den;
}

cudaError_t launch_residual(int n, int Bl, const double *area, const double *rin, const double *stop,
                            const double *sbot, double *scratch, cudaStream_t s) {
    if (n <= 0 || Bl <= 0 || Bl > 32) return cudaErrorInvalidValue;
    k_residual<<<kResidualBlocks, 256, 0, s>>>(n, Bl, area, rin, stop, sbot, scratch + 64);
    k_residual_final<<<1, 32, 0, s>>>(kResidualBlocks, Bl, scratch + 64, scratch);
    return cudaGetLastError();
}

cudaError_t launch_direct_sweep(const SweepDirectParams &p, int max_blocks, cudaStream_t s) {
    const long long total = (long long)p.sc.n * p.dimx * p.dimy * p.nsun;
    if (total <= 0) return cudaSuccess;
    unsigned nb = blocks_for(total, kBlock);
    if ((int)nb > max_blocks) nb = (unsigned)max_blocks;
    k_direct_sweep<<<nb, kBlock, 0, s>>>(p);
    return cudaGetLastError();
}

template <int MINB>
static cudaError_t diffuse_record_b(const DiffuseParams &q, cudaStream_t s) {
    static int blocks_per_sm = 0, sms = 0;
    if (blocks_per_sm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_diffuse_ps<1, true, MINB, false>, kBlock, 0);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    cudaError_t e = cudaMemsetAsync(q.fetch, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    k_diffuse_ps<1, true, MINB, false><<<sms * blocks_per_sm, kBlock, 0, s>>>(q);
    return cudaGetLastError();
}

// variant: DV_PS4 for 4 resident blocks per SM, anything else 3 (the default).
cudaError_t launch_diffuse_record(const DiffuseParams &p, uint32_t *hits, int variant, cudaStream_t s) {
    if ((long long)p.count * p.dimx * p.dimy <= 0) return cudaSuccess;
    DiffuseParams q = p;
    q.hits = hits;
    q.Bc = 1;
    return variant == DV_PS4 ? diffuse_record_b<4>(q, s) : diffuse_record_b<3>(q, s);
}

cudaError_t launch_gather(const GatherParams &p, cudaStream_t s) {
    const int nf = ((p.faces & 1) ? 1 : 0) + ((p.faces & 2) ? 1 : 0);
    const long long warps = (long long)nf * p.n;
    if (warps <= 0) return cudaSuccess;
    long long blocks = (warps * 32 + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    const int cpl = (p.C + 31) / 32;
    if (cpl <= 1) k_gather<1><<<(unsigned)blocks, 256, 0, s>>>(p);
    else if (cpl <= 2) k_gather<2><<<(unsigned)blocks, 256, 0, s>>>(p);
    else if (cpl <= 4) k_gather<4><<<(unsigned)blocks, 256, 0, s>>>(p);
    else if (cpl <= 8) k_gather<8><<<(unsigned)blocks, 256, 0, s>>>(p);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_epilogue_direct_channels(const ChannelEpilogue &p, cudaStream_t s) {
    const long long m = (long long)p.n * p.C;
    if (m <= 0) return cudaSuccess;
    k_epilogue_direct_channels<<<blocks_for(m, 256), 256, 0, s>>>(p, p.C / p.Bl);
    return cudaGetLastError();
}

cudaError_t launch_epilogue_diffuse_channels(const ChannelEpilogue &p, cudaStream_t s) {
    const long long m = (long long)p.n * p.C;
    if (m <= 0) return cudaSuccess;
    k_epilogue_diffuse_channels<<<blocks_for(m, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_copy_channels(int n, int C, const uint8_t *mask, double *src_top, double *src_bot, float *otop,
                                 float *obot, int zero, cudaStream_t s) {
    const long long m = (long long)n * C;
    if (m <= 0) return cudaSuccess;
    k_copy_channels<<<blocks_for(m, 256), 256, 0, s>>>(n, C, mask, src_top, src_bot, otop, obot, zero);
    return cudaGetLastError();
}

cudaError_t launch_fold_channels(int n, int C, const uint8_t *mask, const int8_t *twosided, double *stop,
                                 double *sbot, float *otop, float *obot, cudaStream_t s) {
    const long long m = (long long)n * C;
    if (m <= 0) return cudaSuccess;
    k_fold_channels<<<blocks_for(m, 256), 256, 0, s>>>(n, C, mask, twosided, stop, sbot, otop, obot);
    return cudaGetLastError();
}

}  // namespace hrt
