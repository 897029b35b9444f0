// hrt_trace.cuh -- device-side tracing shared by the trace translation units:
// closest/any-hit traversal of the binary BVH with periodic wrapping, ray origins and
// directions, the sky distribution and the persistent diffuse kernel template.
// Everything is in an unnamed namespace: each including unit gets its own copy.
#pragma once
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

// Translucent-cover query of a launch with covers (sc.cover): mode 0 lets the ray pass
// every cover of its source bit; mode 1 reports only covers after (tlo, ilo) in the order
// (distance, primitive index), never the ray's own origin primitive.
struct CoverQ {
    uint32_t cbit;
    int mode;
    float tlo;
    uint32_t ilo;
    uint32_t self;
};
constexpr int kMaxCovers = 16;  // covers taken per periodic segment of a ray

constexpr int32_t kSentinel = 0x7FFFFFF0;  // no node (empty stack, missed child)
constexpr int kStack4 = 128;               // a 4-wide node pushes up to three children

// Slab offsets of a compressed 4-wide node for a ray: b = (p - o) * inv per axis, p the
// node's lower corner (q0.xyz).
__device__ __forceinline__ f3 node4_offset(const float4 q0, f3 o, f3 inv) {
    return mk((q0.x - o.x) * inv.x, (q0.y - o.y) * inv.y, (q0.z - o.z) * inv.z);
}
// The same from the origin premultiplied (ooi = o * inv), one fused multiply-add per axis:
// b = p * inv - ooi.  Its rounding (of ooi, |o| 2^-24 in space) is of the order of the other
// form's and far inside the leaf-box padding ((|x| + extent) 2^-20) for rays that start in the
// scene, as diffuse rays do.
__device__ __forceinline__ f3 node4_offset_ooi(const float4 q0, f3 ooi, f3 inv) {
    return mk(__fmaf_rn(q0.x, inv.x, -ooi.x), __fmaf_rn(q0.y, inv.y, -ooi.y), __fmaf_rn(q0.z, inv.z, -ooi.z));
}

// The four child boxes of a compressed 4-wide node (q0..q3, format in hrt_device.cuh) against
// a ray (inverse direction inv, node offsets b from node4_offset) within [tmin, tmax]: entry
// distances tk (INFINITY: missed) and child references ck in slot order -- kSentinel for a
// missed child when MARK, else every slot's reference (a hit always has tk <= tmax < INFINITY).
template <bool MARK = true>
__device__ __forceinline__ void node4_children(const float4 q0, const float4 q1, const float4 q2, const float4 q3,
                                               f3 b, f3 inv, float tmin, float tmax, float tk[4], int32_t ck[4]) {
    // near / far plane bytes per axis from the sign of the ray direction: with inv >= 0 the
    // lower plane is entered first (q_lo <= q_hi, fma is monotone)
    const uint32_t nx = inv.x >= 0.f ? __float_as_uint(q1.x) : __float_as_uint(q1.w);
    const uint32_t fx = inv.x >= 0.f ? __float_as_uint(q1.w) : __float_as_uint(q1.x);
    const uint32_t ny = inv.y >= 0.f ? __float_as_uint(q1.y) : __float_as_uint(q2.x);
    const uint32_t fy = inv.y >= 0.f ? __float_as_uint(q2.x) : __float_as_uint(q1.y);
    const uint32_t nz = inv.z >= 0.f ? __float_as_uint(q1.z) : __float_as_uint(q2.y);
    const uint32_t fz = inv.z >= 0.f ? __float_as_uint(q2.y) : __float_as_uint(q1.z);
    const int32_t cref[4] = {__float_as_int(q2.z), __float_as_int(q2.w), __float_as_int(q3.x), __float_as_int(q3.y)};
    // slab planes in the node's quantised frame: t = q * (inv s) + b, one fused multiply-add
    // per plane (inv s is exact: s is a power of two).  The rounding is of the same order as
    // the binary test's and is covered by the leaf-box padding, so no box holding an accepted
    // hit is culled.
    const float ax = inv.x * q0.w, ay = inv.y * q3.z, az = inv.z * q3.w;
    // near and far plane of one axis as one packed pair: the same two subtractions (exact)
    // and fused multiply-adds as the scalar form, in half the instructions
    const unsigned long long bias = f2_pack(8388608.0f, 8388608.0f);
    const unsigned long long ax2 = f2_pack(ax, ax), ay2 = f2_pack(ay, ay), az2 = f2_pack(az, az);
    const unsigned long long bx2 = f2_pack(b.x, b.x), by2 = f2_pack(b.y, b.y), bz2 = f2_pack(b.z, b.z);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float tnx, tfx, tny, tfy, tnz, tfz;
        f2_unpack(f2_fma(f2_sub(f2_pack(q_biased(nx, k), q_biased(fx, k)), bias), ax2, bx2), &tnx, &tfx);
        f2_unpack(f2_fma(f2_sub(f2_pack(q_biased(ny, k), q_biased(fy, k)), bias), ay2, by2), &tny, &tfy);
        f2_unpack(f2_fma(f2_sub(f2_pack(q_biased(nz, k), q_biased(fz, k)), bias), az2, bz2), &tnz, &tfz);
        const float tn = fmax3(tnx, tny, fmaxf(tnz, tmin));
        const float tf = fmin3(tfx, tfy, fminf(tfz, tmax));
        const bool hit = tn <= tf;  // empty slots hold inverted boxes
        tk[k] = hit ? tn : INFINITY;
        ck[k] = (hit || !MARK) ? cref[k] : kSentinel;
    }
}

#define HRT_CSWAP(a, b)                                  \
    if (tk[b] < tk[a]) {                                 \
        const float tt = tk[a];                          \
        tk[a] = tk[b];                                   \
        tk[b] = tt;                                      \
        const int32_t cc = ck[a];                        \
        ck[a] = ck[b];                                   \
        ck[b] = cc;                                      \
    }
// The children of node4_children sorted nearest first (a five-comparator network).
__device__ __forceinline__ void node4_sort(float tk[4], int32_t ck[4]) {
    HRT_CSWAP(0, 1)
    HRT_CSWAP(2, 3)
    HRT_CSWAP(0, 2)
    HRT_CSWAP(1, 3)
    HRT_CSWAP(1, 2)
}
// The nearest child of node4_children moved to slot 0 (a three-comparator tournament); the
// others keep the tournament's order.  The lean trace enters the nearest child and pushes the
// rest: ordering them too (node4_sort) saved 0.4 % of the node visits on the 1 M-triangle
// orchard and cost 2.6 % of the time per diffuse launch.
__device__ __forceinline__ void node4_nearest(float tk[4], int32_t ck[4]) {
    HRT_CSWAP(0, 1)
    HRT_CSWAP(2, 3)
    HRT_CSWAP(0, 2)
}
#undef HRT_CSWAP

// node4_children, sorted nearest first.
__device__ __forceinline__ void node4_test(const float4 q0, const float4 q1, const float4 q2, const float4 q3, f3 o,
                                           f3 inv, float tmin, float tmax, float tk[4], int32_t ck[4]) {
    node4_children(q0, q1, q2, q3, node4_offset(q0, o, inv), inv, tmin, tmax, tk, ck);
    node4_sort(tk, ck);
}

// Closest (or any) hit over the BVH.  Visiting order: both child boxes are
// tested against the current best distance; leaf children are intersected at
// once; of two internal children the nearer is entered and the farther pushed.
// COV: apply the cover query cq to every geometric hit.
template <bool STATS, bool COV = false>
__device__ Hit trace_bvh(const TraceScene &sc, f3 o, f3 d, float tmin, float tmax, bool anyhit, const VoxKey &vk,
                         uint32_t *nv, uint32_t *np, const CoverQ *cq = nullptr) {
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
    uint32_t budget = sc.visit_budget;
    for (;;) {
        if ((uint32_t)cur >= ni || budget-- == 0u) {
            raise(sc.status, budget == 0xFFFFFFFFu ? ERR_BUDGET : ERR_BOUNDS);
            return h;
        }
        if (STATS) ++*nv;
        float4 n0, n1, n2, n3;
        load_node64(sc.nodes, cur, n0, n1, n2, n3);
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
                if (rec_hit(sc.rec, (uint32_t)(~ck), w, o, d, inv, tmin, best, vk, &t, &face, &orig, sc.masks)) {
                    if (COV) {
                        const bool cov = (__ldg(sc.cover + orig) & cq->cbit) != 0u;
                        if (cq->mode == 0 ? cov
                                          : (!cov || orig == cq->self ||
                                             !(t > cq->tlo || (t == cq->tlo && orig > cq->ilo))))
                            continue;
                    }
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

// Closest (or any) hit over the compressed 4-wide nodes (sc.nodes4).  Each visit tests the four
// child boxes against the current best distance and orders them (sorted nearest first, or for an
// any-hit trace only the nearest moved first); leaf children are intersected at once; of the
// internal children the first in that order is entered and the others are pushed, the next in
// order on top.
// The closest hit (ties to the smaller original index) is the binary trace's; an any-hit trace
// may report another occluder.
template <bool STATS>
__device__ Hit trace_bvh4(const TraceScene &sc, f3 o, f3 d, float tmin, float tmax, bool anyhit, const VoxKey &vk,
                          uint32_t *nv, uint32_t *np) {
    Hit h{tmax, 0xFFFFFFFFu, 0};
    if (sc.n == 0) return h;
    WT w = wt_setup(d);
    f3 inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    int32_t stack[kStack4];
    int sp = 0;
    int32_t cur = 0;
    float best = tmax;
    const uint32_t n4 = (uint32_t)sc.n4;
    uint32_t budget = sc.visit_budget;
    for (;;) {
        if ((uint32_t)cur >= n4 || budget-- == 0u) {
            raise(sc.status, budget == 0xFFFFFFFFu ? ERR_BUDGET : ERR_BOUNDS);
            return h;
        }
        if (STATS) ++*nv;
        float4 q0, q1, q2, q3;
        load_node64(sc.nodes4, cur, q0, q1, q2, q3);
        float tk[4];
        int32_t ck[4];
        node4_children(q0, q1, q2, q3, node4_offset(q0, o, inv), inv, tmin, best, tk, ck);
        // an any-hit trace needs only the nearest child first (1.7 ms less per direct pass of
        // the 1 M-triangle orchard than the full sort)
        if (anyhit) node4_nearest(tk, ck);
        else node4_sort(tk, ck);
        // internal children: the lowest slot entered, the others pushed as they come (higher
        // slots first, so the next-lowest is on top) with no array of them to index (which
        // lived in local memory: 4.82 -> 4.64 s per day sweep of the 1 M-triangle orchard);
        // leaf children tested at once
        int32_t nxt = kSentinel;
#pragma unroll
        for (int k = 3; k >= 0; --k) {
            const int32_t c = ck[k];
            if (c == kSentinel) continue;
            if (c >= 0) {
                if (nxt != kSentinel) {
                    if (sp >= kStack4) {
                        raise(sc.status, ERR_STACK);
                        return h;
                    }
                    stack[sp++] = nxt;
                }
                nxt = c;
                continue;
            }
            if ((uint32_t)(~c) >= (uint32_t)sc.n) {
                raise(sc.status, ERR_BOUNDS);
                continue;
            }
            float t;
            int face;
            uint32_t orig;
            if (STATS) ++*np;
            if (rec_hit(sc.rec, (uint32_t)(~c), w, o, d, inv, tmin, best, vk, &t, &face, &orig, sc.masks)) {
                if (h.prim == 0xFFFFFFFFu || t < h.t || (t == h.t && orig < h.prim)) {
                    h.t = t;
                    h.prim = orig;
                    h.face = face;
                    best = t;
                }
                if (anyhit) return h;
            }
        }
        if (nxt == kSentinel) {
            if (sp == 0) break;
            nxt = stack[--sp];
        }
        cur = nxt;
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
// o_last (optional): origin of the last segment traced.  W4: over the compressed 4-wide nodes
// (the caller checks that sc.nodes4 is set).
template <bool STATS, bool W4 = false>
__device__ Hit trace_full(const TraceScene &sc, f3 o, f3 d, float tmin, float tmax, bool anyhit, VoxKey vk,
                          uint32_t *nv, uint32_t *np, f3 *o_last = nullptr) {
    const uint32_t c2 = vk.c2;
    for (int wrap = 0; wrap < 10; ++wrap) {
        vk.c2 = c2 | ((uint32_t)wrap << 16);
        if (o_last) *o_last = o;
        const bool any = anyhit && sc.nbbox == 0;
        Hit h = W4 ? trace_bvh4<STATS>(sc, o, d, tmin, tmax, any, vk, nv, np)
                   : trace_bvh<STATS>(sc, o, d, tmin, tmax, any, vk, nv, np);
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

// trace_full for a launch with covers (OptiX8DeviceCode.cu:816-911 any-hit semantics, made
// deterministic): the closest opaque hit with every cover of source bit `cbit` passed, then,
// when `collect`, the covers of each periodic segment before its end in the order
// (distance, primitive index), each reported to on_cover(prim, face).
template <class F>
__device__ Hit trace_covers(const TraceScene &sc, f3 o, f3 d, float tmin, float tmax, VoxKey vk, uint32_t cbit,
                            uint32_t self, bool collect, F &&on_cover) {
    const uint32_t c2 = vk.c2;
    const CoverQ q0{cbit, 0, -1.f, 0u, self};
    for (int wrap = 0; wrap < 10; ++wrap) {
        vk.c2 = c2 | ((uint32_t)wrap << 16);
        Hit h = trace_bvh<false, true>(sc, o, d, tmin, tmax, false, vk, nullptr, nullptr, &q0);
        const float lim = (h.prim != 0xFFFFFFFFu) ? h.t : tmax;
        float tb = lim;
        int which = -1;
        const bool wall = sc.nbbox > 0 && wall_closest(sc, o, d, tmin, lim, &tb, &which) &&
                          (h.prim == 0xFFFFFFFFu || tb < h.t);
        if (collect) {
            CoverQ q1{cbit, 1, -1.f, 0u, self};
            const float end = wall ? tb : lim;
            for (int c = 0; c < kMaxCovers; ++c) {
                const Hit g = trace_bvh<false, true>(sc, o, d, tmin, end, false, vk, nullptr, nullptr, &q1);
                if (g.prim == 0xFFFFFFFFu) break;
                on_cover(g.prim, g.face);
                q1.tlo = g.t;
                q1.ilo = g.prim;
            }
        }
        if (!wall) return h;
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
    return Hit{tmax, kLost, 0};
}

// A cover's absorbed and reflected shares of `incoming` for launched band b at sheet optics
// (tau, rho, alpha): reflection leaves from the face the ray arrived on
// (OptiX8DeviceCode.cu:874-895).
__device__ __forceinline__ void cover_deposit(const GlassParams &gl, uint32_t c, int face, int b, double incoming,
                                              float rho, float alpha) {
    if (!(incoming > 0.0)) return;
    const size_t i = (size_t)c * gl.Bl + b;
    atomicAdd(gl.rin + i, incoming * (double)alpha);
    atomicAdd((face ? gl.stop : gl.sbot) + i, incoming * (double)rho);
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
// Origins on masked primitives avoid transparent texels (OptiX8DeviceCode.cu:1252-1308):
// up to ten redraws, uniform over the primitive, from Philox counters
// (r, p, c2, 2^31 | attempt); the tenth redraw is kept unchecked, as in the reference.
__device__ __noinline__ void mask_origin(const MaskSet &ms, uint32_t type, uint32_t r, uint32_t p, uint32_t c2,
                                         uint32_t seed, uint32_t pass, float *uu, float *vv) {
    for (uint32_t a = 0; a < 10; ++a) {
        float fu, fv;
        if (type == PT_TRI) {
            const float lo = *uu < *vv ? *uu : *vv, hi = *uu < *vv ? *vv : *uu;
            tri_uv(ms, p, hi - lo, lo, &fu, &fv);
        } else {
            patch_uv(ms, p, *uu - 0.5f, *vv - 0.5f, &fu, &fv);
        }
        if (mask_opaque(ms, ms.id[p], fu, fv)) return;
        const u4 q = philox(r, p, c2, 0x80000000u | (a + 1u), seed, pass);
        *uu = u01(q.a);
        *vv = u01(q.b);
    }
}

__device__ __forceinline__ bool masked_origin(const MaskSet &ms, uint32_t type, uint32_t p) {
    return ms.id && (type == PT_PATCH || type == PT_TILE || type == PT_TRI) && ms.id[p] >= 0;
}

__device__ __forceinline__ f3 direct_origin(const float4 g[4], uint32_t type, uint32_t r, uint32_t p, uint32_t c2,
                                            int dimx, int dimy, uint32_t seed, uint32_t pass, const u4 &u,
                                            const MaskSet &ms) {
    float uu = u01(u.a), vv = u01(u.b), ww = 0.f;
    if (type != PT_TRI) {
        const int xi = (int)(r % (uint32_t)dimx), yi = (int)(r / (uint32_t)dimx);
        uu = ((float)xi + uu) / (float)dimx;
        vv = ((float)yi + vv) / (float)dimy;
    }
    if (masked_origin(ms, type, p)) mask_origin(ms, type, r, p, c2, seed, pass, &uu, &vv);
    if (type == PT_VOXEL) ww = u01(philox(r, p, c2 | 1u, 0u, seed, pass).a);
    return sample_point(g, type, uu, vv, ww);
}

// Origin and direction of diffuse ray r of primitive p from face `face` (1 top, 0
// bottom).  Surfaces: cosine-weighted about the normal, counter (r, p, face, 0).  Voxels
// (VOX builds only): both faces share the sample of counter (r, p, 1, 0), the third
// coordinate comes from (r, p, 2, 0), and the bottom face flips the direction.
// diffuse_ray with the ray's stratum given: ti = r % dimx, pi = r / dimx.
template <bool VOX>
__device__ __forceinline__ void diffuse_ray_cell(const float4 g[4], uint32_t type, uint32_t r, uint32_t p, int face,
                                                 int ti, int pi, int dimx, int dimy, uint32_t seed, uint32_t pass,
                                                 f3 *org, f3 *dir, const MaskSet &ms) {
    f3 dd;
    if (VOX && type == PT_VOXEL) {
        const u4 u = philox(r, p, 1u, 0u, seed, pass);
        const float w = u01(philox(r, p, 2u, 0u, seed, pass).a);
        dd = voxel_dir(ti, pi, dimx, dimy, u01(u.a), u01(u.b));
        *org = sample_point(g, type, u01(u.c), u01(u.d), w);
    } else {
        const u4 u = philox(r, p, (uint32_t)face, 0u, seed, pass);
        dd = diffuse_dir(xyz(g[3]), ti, pi, dimx, dimy, u01(u.a), u01(u.b));
        float uu = u01(u.c), vv = u01(u.d);
        if (masked_origin(ms, type, p)) mask_origin(ms, type, r, p, (uint32_t)face, seed, pass, &uu, &vv);
        *org = sample_point(g, type, uu, vv, 0.f);
    }
    *dir = (face == 0) ? mk(-dd.x, -dd.y, -dd.z) : dd;
}
template <bool VOX>
__device__ __forceinline__ void diffuse_ray(const float4 g[4], uint32_t type, uint32_t r, uint32_t p, int face,
                                            int dimx, int dimy, uint32_t seed, uint32_t pass, f3 *org, f3 *dir,
                                            const MaskSet &ms) {
    diffuse_ray_cell<VOX>(g, type, r, p, face, (int)(r % (uint32_t)dimx), (int)(r / (uint32_t)dimx), dimx, dimy,
                          seed, pass, org, dir, ms);
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

// Refill threshold of the persistent trace (DiffuseParams::refill): a warp leaves the node
// loop when fewer than 8 of its lanes are still in it, so that lanes whose rays ended take new
// ones (Aila & Laine 2009, dynamic ray fetch); the interrupted rays resume where they were.
// Measured on the 1 M-triangle orchard (4-wide trace, per diffuse launch): off 251 ms, 4 232 ms,
// 8 229 ms, 16 240 ms, 28 283 ms.  Scenes with voxels keep it off: on the deep-scatter scene the
// 4-wide trace took 80.5 ms with it against 78.1 ms without.  HRT_REFILL overrides (0-32).
constexpr int kRefillDefault = 8;
// The lean 4-wide trace (hrt_trace_w4.cuh) keeps fewer registers per lane and refills more
// cheaply; on the same workload, per diffuse launch, with two postponed leaves and no leaf
// vote: 8 162.5 ms, 10 160.4 ms, 12 160.2 ms, 14 161.2 ms, 16 162.7 ms, 18 161.8 ms, 20 161.1 ms,
// 24 170.6 ms (run to run on one box within 0.02 ms).
constexpr int kRefillLean = 12;
inline int refill_threshold(bool voxels, bool lean = false) {
    static const int env = [] {  // initialised once, thread-safe; -1: not set
        const char *e = getenv("HRT_REFILL");
        const int v = e ? atoi(e) : -1;
        return (v < -1 || v > 32) ? -1 : v;
    }();
    if (env >= 0) return env;
    return voxels ? 0 : (lean ? kRefillLean : kRefillDefault);
}

// Blocks of a persistent launch: one resident wave; with a lane budget, enough blocks
// that every ray id is taken even if each lane takes exactly its budget (the hardware
// starts the extra blocks as earlier ones retire).
inline unsigned ps_grid(const DiffuseParams &p, int resident) {
    if (!p.lane_budget) return (unsigned)resident;
    const unsigned long long nf = ((p.faces & 1) ? 1 : 0) + ((p.faces & 2) ? 1 : 0);
    const unsigned long long total = (unsigned long long)p.count * (unsigned long long)(p.dimx * p.dimy) * nf;
    const unsigned long long per_block = (unsigned long long)kBlock * p.lane_budget;
    unsigned long long g = (total + per_block - 1) / per_block;
    if (g < (unsigned long long)resident) g = (unsigned long long)resident;
    if (g > 0x7FFFFFFFull) g = 0x7FFFFFFFull;
    return (unsigned)g;
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

// MINB: resident blocks per SM the register allocation must allow (4, the default: 64
// registers; 3: more registers, fewer warps).  VOX: the scene holds voxels (turbid media
// with their own ray sampling); without it the voxel code is left out.
template <int NB, bool RECORD, int MINB, bool VOX, bool W4, bool STATS>
__global__ void __launch_bounds__(kBlock, MINB) k_diffuse_ps(const DiffuseParams P) {
    unsigned long long *fetch = P.fetch;
    const int lane = threadIdx.x & 31;
    const uint32_t R = (uint32_t)(P.dimx * P.dimy);
    // count x R x faces < 2^31: the host splits larger passes into primitive chunks
    const uint32_t per_face = P.count * R;
    const int nf = ((P.faces & 1) ? 1 : 0) + ((P.faces & 2) ? 1 : 0);
    const unsigned long long total = (unsigned long long)per_face * (unsigned long long)nf;
    const uint32_t ni = (uint32_t)(P.sc.n > 1 ? P.sc.n - 1 : 1);
    const uint32_t n4 = (uint32_t)P.sc.n4;
    uint32_t nvis = 0, ntest = 0;  // statistics builds only
    const TraceScene &sc = P.sc;

    bool live = false, exhausted = false;
    f3 o = mk(0.f, 0.f, 0.f), d = o, inv = o, ooi = o;
    WT w = wt_setup(mk(0.f, 0.f, 1.f));
    float best = 1e38f;
    uint32_t bprim = 0xFFFFFFFFu;
    int bface = 0;
    int32_t cur = kSentinel, leaf = 0;
    int sp = 0;
    int32_t stack[W4 ? kStack4 : kStack];
#define POP() (sp > 0 ? stack[--sp] : kSentinel)
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

    uint32_t taken = 0;
    for (;;) {
        // ---- refill lanes without a ray; a lane that has taken its budget retires, so
        // that the block exits and the SM can run blocks of other launches in between
        if (!live && P.lane_budget && taken >= P.lane_budget) exhausted = true;
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
                    ++taken;
                    const uint32_t fi = (uint32_t)(id / per_face);
                    const uint32_t rem = (uint32_t)(id - (unsigned long long)fi * per_face);
                    face = (nf == 2) ? (fi == 0 ? 1 : 0) : ((P.faces & 1) ? 1 : 0);
                    p = P.offset + rem / R;
                    const uint32_t r = rem % R;
                    // recorded hits are laid out [face][primitive][ray] over the whole scene,
                    // whatever primitive chunk this launch covers
                    if (RECORD) rid = ((unsigned long long)fi * (unsigned long long)sc.n + p) * R + r;
                    const int ts = sc.twosided[p];
                    const bool skip = (face == 1 && ts == 3) || (face == 0 && ts != 1);
                    if (!skip) {
                        float4 g[4];
                        load_rgen(sc, p, g);
                        const uint32_t type = __float_as_uint(g[0].w);
                        diffuse_ray<VOX>(g, type, r, p, face, P.dimx, P.dimy, P.seed, P.pass, &o, &d, sc.masks);
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
                        budget = sc.visit_budget;
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
        if (W4) {
            // compressed 4-wide nodes: test the four decoded child boxes, push the hit
            // children farthest first and continue with the nearest
            while (cur >= 0 && cur != kSentinel) {
                if ((uint32_t)cur >= n4 || budget-- == 0u) {
                    raise(sc.status, budget == 0xFFFFFFFFu ? ERR_BUDGET : ERR_BOUNDS);
                    cur = kSentinel;
                    leaf = 0;
                    break;
                }
                if (STATS) ++nvis;
                float4 q0, q1, q2, q3;
                load_node64(sc.nodes4, cur, q0, q1, q2, q3);
                float tk[4];
                int32_t ck[4];
                node4_test(q0, q1, q2, q3, o, inv, 1e-4f, best, tk, ck);
                if (ck[0] == kSentinel) {
                    cur = POP();
                } else {
                    if (sp + 3 > kStack4) {
                        raise(sc.status, ERR_STACK);
                        cur = kSentinel;
                        leaf = 0;
                        break;
                    }
#pragma unroll
                    for (int k = 3; k >= 1; --k)
                        if (ck[k] != kSentinel) stack[sp++] = ck[k];
                    cur = ck[0];
                }
                if (cur < 0 && leaf == 0) {
                    leaf = cur;
                    cur = POP();
                }
                const unsigned am = __activemask();
                if (__all_sync(am, leaf != 0) || __popc(am) < P.refill) break;
            }
        } else {
            while (cur >= 0 && cur != kSentinel) {
                if ((uint32_t)cur >= ni || budget-- == 0u) {
                    raise(sc.status, budget == 0xFFFFFFFFu ? ERR_BUDGET : ERR_BOUNDS);
                    cur = kSentinel;
                    leaf = 0;
                    break;
                }
                if (STATS) ++nvis;
                float4 n0, n1, n2, n3;
                load_node64(sc.nodes, cur, n0, n1, n2, n3);
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
                const unsigned am = __activemask();
                if (__all_sync(am, leaf != 0) || __popc(am) < P.refill) break;
            }
        }
        // ---- primitive tests
        while (leaf != 0) {
            const uint32_t slot = (uint32_t)(~leaf);
            if (STATS) ++ntest;
            if (slot < (uint32_t)sc.n) {
                float t;
                int fc;
                uint32_t orig;
                const VoxKey vk{rr, p, (uint32_t)face | ((uint32_t)wraps << 16), P.seed, P.pass};
                if (rec_hit<VOX>(sc.rec, slot, w, o, d, inv, 1e-4f, best, vk, &t, &fc, &orig, sc.masks)) {
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
                cur = POP();
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
                    budget = sc.visit_budget;
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
    if (STATS && sc.visits) {
        atomicAdd(sc.visits, (unsigned long long)nvis);
        atomicAdd(sc.visits + 1, (unsigned long long)ntest);
    }
#undef POP
#undef ACC
}

}  // namespace

}  // namespace hrt
