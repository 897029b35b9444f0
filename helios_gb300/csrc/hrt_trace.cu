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
#include "hrt_trace.cuh"

namespace hrt {

namespace {

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

// W4: shadow rays over the compressed 4-wide nodes (sc.nodes4 set), else the binary nodes.
template <bool STATS, bool W4>
__global__ void __launch_bounds__(kBlock, 3) k_direct(const DirectParams P) {
    const uint32_t R = (uint32_t)(P.dimx * P.dimy);
    const uint32_t total = P.count * R;  // < 2^31: the host plans primitive chunks
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
                f3 org = direct_origin(g, type, r, p, c2, P.dimx, P.dimy, P.seed, P.pass, u, P.sc.masks);
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
                        Hit h = trace_full<STATS, W4>(P.sc, org, dir, 1e-4f, tmax, true,
                                                      VoxKey{r, p, c2, P.seed, P.pass}, &nv, &np);
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

template <int NB, bool STATS>
__global__ void __launch_bounds__(kBlock) k_diffuse(const DiffuseParams P) {
    const uint32_t R = (uint32_t)(P.dimx * P.dimy);
    const uint32_t total = P.count * R;  // < 2^31: the host plans primitive chunks
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
            diffuse_ray<true>(g, type, r, p, face, P.dimx, P.dimy, P.seed, P.pass, &org, &dir, P.sc.masks);
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

// ------------------------------------------------------ translucent covers --
// Launches whose scene holds covers (glass in every launched band; sc.cover) run these
// one-ray-per-thread kernels: the ray passes every cover of its source, each cover crossed
// before the ray's end attenuates it by the sheet transmittance per band and takes its
// absorbed and reflected shares of the flux reaching it (OptiX8DeviceCode.cu:816-911), and
// only sky or source deposits see the attenuation (:542, :630).

// incidence cosine of direction d on primitive c (unit normal of its ray-origin record)
__device__ __forceinline__ float cover_cos(const TraceScene &sc, uint32_t c, f3 d) {
    const float4 n = __ldg(sc.rgen + 4 * (size_t)c + 3);
    return fminf(1.f, fabsf(dot(d, xyz(n))));
}

__global__ void __launch_bounds__(kBlock) k_direct_glass(const DirectParams P) {
    const uint32_t R = (uint32_t)(P.dimx * P.dimy);
    const uint32_t total = P.count * R;  // < 2^31: the host plans primitive chunks
    const uint32_t stride = gridDim.x * blockDim.x;
    const double inv_nr = 1.0 / (double)R;
    const GlassParams &gl = P.gl;
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
            double v[2] = {0.0, 0.0};
            bool live = active;
            if (live) {
                const uint32_t c2 = (uint32_t)(k << 1);
                u4 u = philox(r, p, c2, 0u, P.seed, P.pass);
                const bool vox = type == PT_VOXEL;
                f3 org = direct_origin(g, type, r, p, c2, P.dimx, P.dimy, P.seed, P.pass, u, P.sc.masks);
                f3 nrm = xyz(g[3]);
                f3 dir;
                float tmax;
                double strength;
                live = direct_ray(P.src[k], org, nrm, vox, u.c, u.d, inv_nr, &dir, &tmax, &strength);
                if (live) {
                    const int face = (vox || dot(dir, nrm) > 0.f) ? 1 : 0;
                    if ((!face && ts == 0) || ts == 3) {
                        live = false;
                    } else {
                        float T[kGlassBands];
#pragma unroll
                        for (int b = 0; b < kGlassBands; ++b) T[b] = 1.f;
                        bool crossed = false;
                        Hit h = trace_covers(P.sc, org, dir, 1e-4f, tmax, VoxKey{r, p, c2, P.seed, P.pass}, 1u << k, p,
                                             true, [&](uint32_t c, int cface) {
                                                 crossed = true;
                                                 const float cs = cover_cos(P.sc, c, dir);
                                                 int b = -1;
                                                 for (int bg = 0; bg < gl.Bg && b + 1 < kGlassBands; ++bg) {
                                                     if (!gl.flags[bg]) continue;
                                                     ++b;
                                                     const size_t m = ((size_t)k * P.sc.n + c) * gl.Bg + bg;
                                                     float tc, rc, ac;
                                                     glass_trs(cs, gl.gn[m], gl.gkl[m], &tc, &rc, &ac);
                                                     cover_deposit(gl, c, cface, b,
                                                                   strength * (double)gl.src_flux[k * gl.Bl + b] *
                                                                       (double)T[b],
                                                                   rc, ac);
                                                     T[b] *= tc;
                                                 }
                                             });
                        if (h.prim == 0xFFFFFFFFu) {
                            if (!crossed) {
                                v[face] = strength;
                            } else {
                                double *dst = gl.Gcov + (((size_t)p * P.S + k) * 2 + face) * gl.Bl;
                                int b = -1;
                                for (int bg = 0; bg < gl.Bg && b + 1 < kGlassBands; ++bg) {
                                    if (!gl.flags[bg]) continue;
                                    ++b;
                                    atomicAdd(dst + b, strength * (double)T[b]);
                                }
                            }
                        }
                    }
                }
            }
            count_rays(P.sc, live);
            uint32_t key = active ? (p * (uint32_t)P.S + (uint32_t)k) : 0xFFFFFFFFu;
            warp_segment_add<2>(key, v, 2, P.G, 2);
        }
    }
}

template <int NB>
__global__ void __launch_bounds__(kBlock) k_diffuse_glass(const DiffuseParams P) {
    const uint32_t R = (uint32_t)(P.dimx * P.dimy);
    const uint32_t total = P.count * R;  // < 2^31: the host plans primitive chunks
    const uint32_t stride = gridDim.x * blockDim.x;
    const int face = (blockIdx.y == 0) ? 1 : 0;
    if (!(P.faces & (1 << blockIdx.y))) return;
    double *G = face ? P.Gt : P.Gb;
    const double inv_r = 1.0 / (double)R;
    const GlassParams &gl = P.gl;
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
        if (active) {
            float4 g[4];
            load_rgen(P.sc, p, g);
            uint32_t type = __float_as_uint(g[0].w);
            f3 org, dir;
            diffuse_ray<true>(g, type, r, p, face, P.dimx, P.dimy, P.seed, P.pass, &org, &dir, P.sc.masks);
            float T[NB];
#pragma unroll
            for (int j = 0; j < NB; ++j) T[j] = 1.f;
            // covers take the launch's isotropic sky flux (OptiX8DeviceCode.cu:871-880)
            Hit h = trace_covers(P.sc, org, dir, 1e-4f, 1e38f, VoxKey{r, p, (uint32_t)face, P.seed, P.pass}, 1u, p,
                                 gl.sky != 0, [&](uint32_t c, int cface) {
                                     const float cs = cover_cos(P.sc, c, dir);
                                     int b = -1;
                                     for (int bg = 0; bg < gl.Bg && b + 1 < NB; ++bg) {
                                         if (!gl.flags[bg]) continue;
                                         ++b;
                                         const size_t m = (size_t)c * gl.Bg + bg;
                                         float tc, rc, ac;
                                         glass_trs(cs, gl.gn[m], gl.gkl[m], &tc, &rc, &ac);
                                         cover_deposit(gl, c, cface, b, inv_r * (double)P.sky.flux[b] * (double)T[b],
                                                       rc, ac);
                                         T[b] *= tc;
                                     }
                                 });
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
                        if (fl > 0.f) v[j] = sky_fd(dir, P.sky, j) * (double)fl * (double)T[j];
                    }
            }
        }
        count_rays(P.sc, active);
        uint32_t key = active ? p : 0xFFFFFFFFu;
        warp_segment_add<NB>(key, v, P.Bc, G, P.Bl);
    }
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
        org = direct_origin(g, type, r, p, (uint32_t)face, dimx, dimy, seed, pass, u, sc.masks);
        dir = normalize(mk(dx, dy, dz));
    } else {
        diffuse_ray<true>(g, type, r, p, face, dimx, dimy, seed, pass, &org, &dir, sc.masks);
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
        if (P.Gcov) {
            g0 += P.Gcov[(((size_t)p * P.S + s) * 2) * P.Bl + b] * flux;
            g1 += P.Gcov[(((size_t)p * P.S + s) * 2 + 1) * P.Bl + b] * flux;
        }
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
// are exactly those of a plain direct pass with the same seed (source slot 0).  W4: shadow rays
// over the compressed 4-wide nodes (sc.nodes4 set), else the binary nodes.
template <bool W4>
__global__ void __launch_bounds__(kBlock, 3) k_direct_sweep(const SweepDirectParams P) {
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
            const f3 org = direct_origin(g, type, r, p, 0u, P.dimx, P.dimy, P.seed, 0u, u, P.sc.masks);
            const f3 nrm = xyz(g[3]);
            const f3 dd = normalize(mk(P.sun_dir[3 * sun], P.sun_dir[3 * sun + 1], P.sun_dir[3 * sun + 2]));
            const double strength = inv_nr * (double)fabsf(dot(nrm, dd));
            const bool face = dot(dd, nrm) > 0.f;
            if (!((!face && ts == 0) || ts == 3)) {
                live = true;
                uint32_t nv = 0, np = 0;
                const Hit h =
                    trace_full<false, W4>(P.sc, org, dd, 1e-4f, 1e38f, true, VoxKey{r, p, 0u, P.seed, 0u}, &nv, &np);
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
// radiation_out[hit][0..C) (coalesced); a miss adds the channel's sky flux.  The hit codes come
// 32 at a time in one coalesced load and are broadcast by shuffles, so the row loads of
// consecutive hits do not wait on one another.  Sums are compensated FP32 (Kahan: each add
// carries its rounding error into the next), converted to FP64 once per channel: GB300 runs
// FP32 adds at many times its FP64 rate, and the FP64 form of this gather (an F2F and a DADD
// per channel and hit) was FP64-bound at 0.37 s per pass of the 1 M-triangle orchard's day
// sweep.  The compensated sum's error is about 2^-23 of the sum of the values (all >= 0).
template <int CPL>
__global__ void __launch_bounds__(256) k_gather(const GatherParams P) {
    const int lane = threadIdx.x & 31;
    const int nf = ((P.faces & 1) ? 1 : 0) + ((P.faces & 2) ? 1 : 0);
    const long long items = (long long)nf * P.n;
    const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
    float sky[CPL];
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
        const int c = lane + 32 * k;
        sky[k] = c < P.C ? __ldg(P.sky + c) : 0.f;
    }
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
        float sum[CPL], err[CPL];
#pragma unroll
        for (int k = 0; k < CPL; ++k) sum[k] = err[k] = 0.f;
        const uint32_t *row = P.hits + ((size_t)fi * P.n + p) * P.R;
        for (int r0 = 0; r0 < P.R; r0 += 32) {
            const uint32_t mine = (r0 + lane < P.R) ? __ldg(row + r0 + lane) : kLostCode;
            const int nr = min(32, P.R - r0);
#pragma unroll 4
            for (int j = 0; j < nr; ++j) {
                const uint32_t h = __shfl_sync(0xffffffffu, mine, j);  // the same code in every lane
                if (h == kLostCode) continue;
                const bool miss = h == kMissCode;
                const uint32_t hc = miss ? 0u : h;  // a miss reads the sky; its row pointer stays in bounds
                const float *src = ((hc & 1u) ? P.otop : P.obot) + (size_t)(hc >> 1) * P.C;
#pragma unroll
                for (int k = 0; k < CPL; ++k) {
                    const int c = lane + 32 * k;
                    if (c < P.C) {
                        const float x = miss ? sky[k] : __ldg(src + c);
                        const float y = x - err[k], t = sum[k] + y;
                        err[k] = (t - sum[k]) - y;
                        sum[k] = t;
                    }
                }
            }
        }
        double *G = (face ? P.Gt : P.Gb) + (size_t)p * P.C;
#pragma unroll
        for (int k = 0; k < CPL; ++k) {
            const int c = lane + 32 * k;
            if (c < P.C) G[c] = (double)sum[k] - (double)err[k];
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
    if (p.sc.nodes4) k_direct<STATS, true><<<nb, kBlock, 0, s>>>(p);
    else k_direct<STATS, false><<<nb, kBlock, 0, s>>>(p);
    return cudaGetLastError();
}

// Default diffuse variant: the persistent 4-wide traversal; HRT_TRAVERSAL=simple selects
// the one-ray-per-thread kernel and HRT_TRAVERSAL=bvh2 the persistent binary traversal.
static int default_variant() {
    static const int v = [] {  // initialised once, thread-safe
        const char *e = getenv("HRT_TRAVERSAL");
        return (e && e[0] == 's') ? DV_SIMPLE : ((e && e[0] == 'b') ? DV_PS4 : DV_W4);
    }();
    return v;
}

// variant: one of DiffuseVariant (hrt_internal.h); DV_DEFAULT resolves to default_variant().
template <bool STATS>
static cudaError_t diffuse_impl(const DiffuseParams &p, int variant, int max_blocks, cudaStream_t s) {
    int64_t total = (int64_t)p.count * p.dimx * p.dimy;
    if (total <= 0 || p.Bc <= 0) return cudaSuccess;
    if (variant == DV_DEFAULT) variant = default_variant();
    if ((variant == DV_W4 || variant == DV_W43 || is_w4s_variant(variant)) && !p.sc.nodes4) variant = DV_PS4;
    if (is_w4s_variant(variant) && p.sc.voxels) variant = DV_W4;  // the lean kernel has no voxel code
    if (p.fetch && variant != DV_SIMPLE) {
        if (STATS) {
            if (p.Bc <= 4 && is_w4s_variant(variant)) return launch_w4s_stats(p, variant, s);
            if (p.Bc <= 4 && (variant == DV_W4 || variant == DV_W43)) return launch_ps_stats(p, s);
        } else if (p.sc.voxels) {
            return launch_ps_voxels(p, variant, s);
        } else if (is_w4s_variant(variant)) {
            return launch_w4s(p, variant, s);
        } else {
            return launch_ps_accumulate(p, variant, s);
        }
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
cudaError_t launch_direct_glass(const DirectParams &p, int max_blocks, cudaStream_t s) {
    int64_t total = (int64_t)p.count * p.dimx * p.dimy;
    if (total <= 0 || p.S <= 0) return cudaSuccess;
    unsigned nb = blocks_for(total, kBlock);
    if ((int)nb > max_blocks) nb = (unsigned)max_blocks;
    k_direct_glass<<<nb, kBlock, 0, s>>>(p);
    return cudaGetLastError();
}
cudaError_t launch_diffuse_glass(const DiffuseParams &p, int max_blocks, cudaStream_t s) {
    int64_t total = (int64_t)p.count * p.dimx * p.dimy;
    if (total <= 0 || p.Bc <= 0) return cudaSuccess;
    unsigned nb = blocks_for(total, kBlock);
    if ((int)nb > max_blocks) nb = (unsigned)max_blocks;
    dim3 grid(nb, 2);
    if (p.Bc <= 1) k_diffuse_glass<1><<<grid, kBlock, 0, s>>>(p);
    else if (p.Bc <= 4) k_diffuse_glass<4><<<grid, kBlock, 0, s>>>(p);
    else if (p.Bc <= 16) k_diffuse_glass<16><<<grid, kBlock, 0, s>>>(p);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}
cudaError_t launch_diffuse_stats(const DiffuseParams &p, int variant, int max_blocks, cudaStream_t s) {
    return diffuse_impl<true>(p, variant, max_blocks, s);
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
    if (p.sc.nodes4) k_direct_sweep<true><<<nb, kBlock, 0, s>>>(p);
    else k_direct_sweep<false><<<nb, kBlock, 0, s>>>(p);
    return cudaGetLastError();
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
    else if (cpl <= 6) k_gather<6><<<(unsigned)blocks, 256, 0, s>>>(p);
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
