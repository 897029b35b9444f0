// hrt_api.cu -- context, C ABI (include/hrt.h) and the device-resident runBand.
//
// The granular entry points keep the semantics of the reference backend
// (plugins/radiation/src/backends/OptiX8Backend.cpp): launches ACCUMULATE into
// radiation_in / scatter buffers, zero/copy/upload calls do what their
// RayTracingBackend virtuals document.  hrt_run_band() executes the pass
// sequence of RadiationModel::runBand (src/RadiationModel.cpp:3470-4663)
// without returning to the host between passes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hrt.h"
#include "hrt_device.cuh"
#include "hrt_internal.h"

using namespace hrt;

namespace {

// Stream on which buffers being destroyed are released (set by hrt_destroy); without it
// they are released with cudaFree.
thread_local cudaStream_t g_release_stream = nullptr;

// Device buffer of a context.  Allocation is stream-ordered (cudaMallocAsync /
// cudaFreeAsync on the context's stream): cudaMalloc / cudaFree can wait for the whole
// device, which would stall a context behind long kernels of other contexts sharing the
// GPU (the served stream runs many).
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(cudaStream_t s, size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        cap = 0;
        size_t want = bytes ? bytes : 16;
        cudaError_t e = cudaMallocAsync(&p, want, s);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    template <class T>
    T *as() const {
        return (T *)p;
    }
    void free_on(cudaStream_t s) {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        cap = 0;
    }
    void release() {
        if (p) {
            if (g_release_stream) cudaFreeAsync(p, g_release_stream);
            else cudaFree(p);
        }
        p = nullptr;
        cap = 0;
    }
    ~DevBuf() { release(); }
};

// Keep up to 16 GB of freed stream-ordered memory in the device's default pool, so that
// growing a buffer does not unmap and map memory at every synchronisation.
void keep_pool(int device) {
    static std::mutex mu;
    static std::vector<int> done;
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(done.begin(), done.end(), device) != done.end()) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = 16ull << 30;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    done.push_back(device);
}

// Surface area of a primitive in FP64 from its FP32 transform (a voxel's: its leaf area,
// LAD x volume).  Triangles span half the parallelogram of their two edges, disks are
// the unit disk scaled by the transform.
double prim_area(const float *T, uint32_t type, float lad) {
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

}  // namespace

struct hrt_context {
    int device = 0;
    int sms = 152;
    cudaStream_t own = nullptr, stream = nullptr;
    std::string err;
    // geometry
    int n = 0, nbbox = 0;
    float px = 0.f, py = 0.f;
    bool have_geometry = false, built = false;
    std::vector<int8_t> h_twosided;
    std::vector<uint32_t> h_voxels;  // original indices of voxel primitives
    DevBuf T, type, twosided, bbox, rec, rgen, nodes, codes, perm, bvh_scratch, lad, area, nodes4;
    DevBuf mask_id, mask_uv_id, mask_uv, mask_size, mask_offset, mask_data;
    bool masks = false;
    int n4 = 0;  // compressed 4-wide nodes built
    // materials and sources
    int mS = 0, mN = 0, mB = 0;
    DevBuf rho, tau, src, src_flux;
    int S = 0;
    size_t src_flux_count = 0;
    std::vector<float> h_src_flux;
    // radiation buffers
    int Bl = 0;
    DevBuf rin, stop, sbot, otop, obot, ftop, fbot, Gd, Gt, Gb, flags, sky, fin, status, counter, emis, emis_eps, emis_T,
        fetch;
    size_t emis_eps_count = 0, emis_T_count = 0;
    DevBuf io_a, io_b, io_c;  // staging for inspection calls
    uint64_t last_rays = 0, last_kernels = 0, last_iters = 0;
    DevBuf resid;  // scattering residual: block partials and the per-band result
    // measurement: bit 0 counts traversal work, bit 1 times trace launches
    int measure = 0;
    DevBuf visits;
    struct Timed {
        int kind;  // 0 direct, 1 diffuse
        cudaEvent_t a, b;
    };
    std::vector<Timed> timed;
    double meas[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    // batched sweep: inputs, accumulators, recorded hits and the captured graph
    DevBuf sw_in, sw_mat, sw_acc, sw_out, sw_hits;
    cudaGraphExec_t sw_exec = nullptr;
    std::string sw_key;
    int sw_kernels = 0;
    // multi-scene sweeps this context leads: slot tables and the captured graph
    DevBuf sw_slots;
    cudaGraphExec_t mw_exec = nullptr;
    std::string mw_key;
    int mw_kernels = 0;
    unsigned long long multi_rays = 0;
    // rays a lane of the persistent trace takes before its block retires (0: no limit)
    uint32_t lane_budget = 0;
    // rays one trace launch may carry (passes above it run as primitive chunks) and the
    // node-visit budget of a ray segment (0: 2n+64); both lowered only by tests
    uint64_t ray_limit = kLaunchRayLimit;
    uint32_t visit_budget = 0;
    // kernel-variant tuner: choice per pass shape, and a log of the trials
    int tune = 1;
    std::map<std::string, int> tuned;
    std::string tune_log;
    DevBuf tune_g;
    // translucent covers: sheet optics [gS][n][gB] (gS 0: none), the cover bits of the
    // current launch (key: band flags and source count) and the direct pass's per-band sums
    int gS = 0, gB = 0;
    std::vector<int8_t> h_glass;
    DevBuf gn, gkl, cover, Gcov;
    std::string cover_key;
    bool cover_any = false;
    std::vector<uint8_t> h_flags;  // band flags of the current launch
    bool sky_any = false;          // some launched band of the current launch has sky flux
    // cameras: radiance [W*H*Bl] (FP64), labels and depths [W*H], the camera sky model
    // ([sky radiance B][solar disk B][sky flux B][Prague 4B][sun 3B], emission flags [B]) and
    // the camera view of the primitives that hrt_run_band accumulates
    DevBuf cam_pix, cam_lab, cam_dep, cam_sky, cam_em, ctop, cbot;
    int cam_W = 0, cam_H = 0, cam_B = 0, lab_W = 0, lab_H = 0;
    uint32_t cam_id_cur = 0xFFFFFFFFu;
    int sky_B = 0;                 // bands of the camera sky model (0: none)
    bool sky_has[5] = {false, false, false, false, false};  // sky radiance, disk, flux, Prague, emission
    float sky_sun[3] = {0.f, 0.f, 1.f}, sky_cos = 0.f;
    // energy balance: surface arrays (10 x [n] float + [n] sides), R, new temperatures, outputs
    DevBuf eb_surf, eb_sides, eb_R, eb_T, eb_out, eb_status;
    int eb_n = 0;
    float eb_dt = 0.f, eb_Tdef = 300.f;
    uint64_t eb_unconverged = 0;
};

namespace {

int fail(hrt_context *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}
#define CU(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e__ = (call);                                                                  \
        if (e__ != cudaSuccess)                                                                    \
            return fail(ctx, e__ == cudaErrorMemoryAllocation ? HRT_ENOMEM : HRT_ECUDA,            \
                        std::string("CUDA error in ") + #call + ": " + cudaGetErrorString(e__));   \
    } while (0)

TraceScene scene_of(hrt_context *ctx) {
    TraceScene sc;
    sc.rec = ctx->rec.as<float4>();
    sc.nodes = ctx->nodes.as<float4>();
    sc.nodes4 = ctx->n4 > 0 ? ctx->nodes4.as<float4>() : nullptr;
    sc.n4 = ctx->n4;
    sc.rgen = ctx->rgen.as<float4>();
    sc.bbox = ctx->nbbox ? ctx->bbox.as<float4>() : nullptr;
    sc.n = ctx->n;
    sc.nbbox = ctx->nbbox;
    sc.voxels = ctx->h_voxels.empty() ? 0 : 1;
    sc.periodic_x = ctx->px;
    sc.periodic_y = ctx->py;
    sc.twosided = ctx->twosided.as<int8_t>();
    sc.status = ctx->status.as<uint32_t>();
    sc.rays = ctx->counter.as<unsigned long long>();
    sc.visits = (ctx->measure & 1) ? ctx->visits.as<unsigned long long>() : nullptr;
    sc.masks = MaskSet{};
    if (ctx->masks) {
        sc.masks.id = ctx->mask_id.as<int32_t>();
        sc.masks.uv_id = ctx->mask_uv_id.as<int32_t>();
        sc.masks.uv = ctx->mask_uv.as<float>();
        sc.masks.size = ctx->mask_size.as<int32_t>();
        sc.masks.offset = ctx->mask_offset.as<uint32_t>();
        sc.masks.data = ctx->mask_data.as<uint8_t>();
        sc.masks.T = ctx->T.as<float>();
    }
    sc.cover = nullptr;
    const uint64_t vb = 2ull * (uint64_t)std::max(ctx->n, 0) + 64ull;
    sc.visit_budget = ctx->visit_budget ? ctx->visit_budget : (uint32_t)std::min<uint64_t>(vb, 0xFFFFFFFFull);
    return sc;
}

// Primitives per trace launch of a pass with `rays_per_primitive` rays per primitive (all
// faces), or 0 with the context's error set when one primitive's rays exceed a launch.
uint32_t chunk_prims(hrt_context *ctx, uint64_t rays_per_primitive) {
    const uint32_t per = launch_chunk_prims(rays_per_primitive, ctx->ray_limit);
    if (per == 0) fail(ctx, HRT_EUNSUPPORTED, "the rays of one primitive exceed the rays one launch can carry (2^31)");
    return per;
}

int max_blocks(hrt_context *ctx) { return ctx->sms * 8; }

// Launch a trace kernel, bracketed by CUDA events when timing is on.  With traversal counting
// on (statistics launches, untimed), count the launch and the rays it traced instead:
// meas[0] / meas[2] launches, meas[6] / meas[7] rays of direct / diffuse launches.
template <class F>
cudaError_t timed_launch(hrt_context *ctx, int kind, F &&launch) {
    if (ctx->measure & 1) {
        // rays, node visits and primitive tests of this launch: counters before and after
        unsigned long long a = 0, b = 0, va[2] = {0, 0}, vb[2] = {0, 0};
        cudaError_t e = cudaMemcpyAsync(&a, ctx->counter.p, sizeof a, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(va, ctx->visits.p, sizeof va, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = launch();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&b, ctx->counter.p, sizeof b, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(vb, ctx->visits.p, sizeof vb, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return e;
        ctx->meas[kind == 0 ? 0 : 2] += 1.0;
        ctx->meas[kind == 0 ? 6 : 7] += (double)(b - a);
        if (kind != 0) {
            ctx->meas[8] += (double)(vb[0] - va[0]);
            ctx->meas[9] += (double)(vb[1] - va[1]);
        }
        return cudaSuccess;
    }
    if (!(ctx->measure & 2)) return launch();
    hrt_context::Timed t{kind, nullptr, nullptr};
    cudaError_t e = cudaEventCreate(&t.a);
    if (e == cudaSuccess) e = cudaEventCreate(&t.b);
    if (e != cudaSuccess) return e;
    cudaEventRecord(t.a, ctx->stream);
    e = launch();
    cudaEventRecord(t.b, ctx->stream);
    ctx->timed.push_back(t);
    return e;
}

// Fold finished timings into ctx->meas ([0] direct launches, [1] direct ms, [2] diffuse launches, [3] diffuse ms).
void collect_timings(hrt_context *ctx) {
    for (auto &t : ctx->timed) {
        float ms = 0.f;
        if (cudaEventSynchronize(t.b) == cudaSuccess && cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess) {
            ctx->meas[t.kind == 0 ? 0 : 2] += 1.0;
            ctx->meas[t.kind == 0 ? 1 : 3] += ms;
        }
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    ctx->timed.clear();
}

// rotation about x, y, z (reference d_makeTransformMatrix, OptiX8DeviceCode.cu:191-201)
void rotation3(const float r[3], float out[9]) {
    double sx = std::sin((double)r[0]), cx = std::cos((double)r[0]);
    double sy = std::sin((double)r[1]), cy = std::cos((double)r[1]);
    double sz = std::sin((double)r[2]), cz = std::cos((double)r[2]);
    double m[9] = {cz * cy, cz * sy * sx - sz * cx, cz * sy * cx + sz * sx,
                   sz * cy, sz * sy * sx + cz * cx, sz * sy * cx - cz * sx,
                   -sy,     cy * sx,                cy * cx};
    for (int i = 0; i < 9; ++i) out[i] = (float)m[i];
}

int check_built(hrt_context *ctx) {
    if (!ctx->built)
        return fail(ctx, HRT_EINVAL,
                    "No acceleration structure. Call hrt_update_geometry() and hrt_build_accel() before launching rays.");
    return HRT_OK;
}

int sync_and_status(hrt_context *ctx) {
    uint32_t st = 0;
    CU(cudaMemcpyAsync(&st, ctx->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    if (st) {
        CU(cudaMemsetAsync(ctx->status.p, 0, sizeof(uint32_t), ctx->stream));
        char buf[200];
        std::snprintf(buf, sizeof buf, "device error word 0x%x (%s%s%s%s)", st,
                      (st & ERR_STACK) ? "traversal stack overflow " : "", (st & ERR_WRAP) ? "periodic wrap limit " : "",
                      (st & ERR_BOUNDS) ? "index out of range " : "",
                      (st & ERR_BUDGET) ? "traversal visit budget exhausted" : "");
        return fail(ctx, HRT_EDEVICE, buf);
    }
    return HRT_OK;
}

// Radiation buffers for n x Bl values.
int ensure_buffers(hrt_context *ctx, int Bl) {
    size_t m = (size_t)std::max(ctx->n, 1) * (size_t)std::max(Bl, 1);
    CU(ctx->rin.ensure(ctx->stream, m * sizeof(double)));
    CU(ctx->stop.ensure(ctx->stream, m * sizeof(double)));
    CU(ctx->sbot.ensure(ctx->stream, m * sizeof(double)));
    CU(ctx->otop.ensure(ctx->stream, m * sizeof(float)));
    CU(ctx->obot.ensure(ctx->stream, m * sizeof(float)));
    CU(ctx->ftop.ensure(ctx->stream, m * sizeof(double)));
    CU(ctx->fbot.ensure(ctx->stream, m * sizeof(double)));
    CU(ctx->Gt.ensure(ctx->stream, m * sizeof(double)));
    CU(ctx->Gb.ensure(ctx->stream, m * sizeof(double)));
    CU(ctx->fin.ensure(ctx->stream, m * sizeof(float)));
    return HRT_OK;
}

// Device copy of the per-launch sky parameters: [flux Bl][K Bl][norm Bl][peak 3Bl][prague 4Bl].
int upload_sky(hrt_context *ctx, int Bl, const float *flux, const float *K, const float *norm, const float *peak,
               const float *prague, SkyParams *sp) {
    size_t Bn = (size_t)std::max(Bl, 1);
    std::vector<float> h(10 * Bn, 0.f);
    for (int b = 0; b < Bl; ++b) {
        h[b] = flux ? flux[b] : 0.f;
        h[Bn + b] = K ? K[b] : 0.f;
        h[2 * Bn + b] = norm ? norm[b] : 1.f;
        for (int k = 0; k < 3; ++k) h[3 * Bn + 3 * b + k] = peak ? peak[3 * b + k] : (k == 2 ? 1.f : 0.f);
        for (int k = 0; k < 4; ++k) h[6 * Bn + 4 * b + k] = prague ? prague[4 * b + k] : 0.f;
    }
    ctx->sky_any = false;
    for (int b = 0; b < Bl; ++b) ctx->sky_any = ctx->sky_any || h[b] > 0.f;
    CU(ctx->sky.ensure(ctx->stream, h.size() * sizeof(float)));
    CU(cudaMemcpyAsync(ctx->sky.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    float *d = ctx->sky.as<float>();
    sp->flux = d;
    sp->K = d + Bn;
    sp->knorm = d + 2 * Bn;
    sp->peak = d + 3 * Bn;
    sp->prague = d + 6 * Bn;
    return HRT_OK;
}

int upload_flags(hrt_context *ctx, int Bg, const uint8_t *flags) {
    ctx->h_flags.assign(flags, flags + Bg);
    CU(ctx->flags.ensure(ctx->stream, (size_t)std::max(Bg, 1)));
    CU(cudaMemcpyAsync(ctx->flags.p, flags, (size_t)Bg, cudaMemcpyHostToDevice, ctx->stream));
    return HRT_OK;
}

void strata(uint32_t rpp, int *dimx, int *dimy) {
    int dx = (int)std::sqrt((float)rpp);
    *dimx = dx;
    *dimy = dx > 0 ? (int)(rpp / (uint32_t)dx) : 1;
}

// Cover bits of the current launch for rays of sources 0..nsrc-1: bit k of primitive p when p
// is glass for source k in every launched band (RadiationModel.cpp:2759-2807 materials,
// OptiX8DeviceCode.cu:838-850 rule); voxels never are.  *out stays null when no primitive is
// a cover (the launch then runs the ordinary kernels).
int covers_for(hrt_context *ctx, int Bg, int nsrc, const uint32_t **out) {
    *out = nullptr;
    if (ctx->gS == 0) return HRT_OK;
    if (ctx->gB != Bg || ctx->h_glass.size() != (size_t)ctx->gS * ctx->n * ctx->gB)
        return fail(ctx, HRT_EINVAL, "translucent-cover arrays do not match the geometry or bands; call hrt_update_glass()");
    std::string key(ctx->h_flags.begin(), ctx->h_flags.end());
    key += ":" + std::to_string(nsrc);
    if (key != ctx->cover_key) {
        const int n = ctx->n, ns = std::min(std::min(nsrc, ctx->gS), 32);
        std::vector<uint8_t> vox((size_t)n, 0);
        for (uint32_t v : ctx->h_voxels) vox[v] = 1;
        std::vector<uint32_t> bits((size_t)std::max(n, 1), 0u);
        bool any = false;
        for (int p = 0; p < n; ++p) {
            if (vox[p]) continue;
            for (int k = 0; k < ns; ++k) {
                bool launched = false, all = true;
                for (int bg = 0; bg < Bg && all; ++bg) {
                    if (!ctx->h_flags[bg]) continue;
                    launched = true;
                    all = ctx->h_glass[((size_t)k * n + p) * Bg + bg] != 0;
                }
                if (launched && all) {
                    bits[p] |= 1u << k;
                    any = true;
                }
            }
        }
        if (any) {
            CU(ctx->cover.ensure(ctx->stream, bits.size() * sizeof(uint32_t)));
            CU(cudaMemcpyAsync(ctx->cover.p, bits.data(), bits.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                               ctx->stream));
        }
        ctx->cover_any = any;
        ctx->cover_key = key;
    }
    if (ctx->cover_any) *out = ctx->cover.as<uint32_t>();
    return HRT_OK;
}

GlassParams glass_params(hrt_context *ctx, int Bg, int Bl) {
    GlassParams g{};
    g.gn = ctx->gn.as<float>();
    g.gkl = ctx->gkl.as<float>();
    g.flags = ctx->flags.as<uint8_t>();
    g.Bg = Bg;
    g.Bl = Bl;
    g.sky = ctx->sky_any ? 1 : 0;
    g.rin = ctx->rin.as<double>();
    g.stop = ctx->stop.as<double>();
    g.sbot = ctx->sbot.as<double>();
    return g;
}

// Direct pass + epilogue (__raygen__direct / __miss__direct).
int direct_pass(hrt_context *ctx, uint32_t offset, uint32_t count, uint32_t rpp, uint32_t seed, uint32_t pass, int Bg,
                int Bc, int Bl) {
    int dimx, dimy;
    strata(rpp, &dimx, &dimy);
    if (dimx * dimy == 0 || count == 0 || ctx->S == 0) return HRT_OK;
    if (ctx->mS < ctx->S || ctx->mN != ctx->n)
        return fail(ctx, HRT_EINVAL, "materials do not match the geometry/sources; call hrt_update_materials()");
    if (ctx->src_flux_count < (size_t)ctx->S * Bl)
        return fail(ctx, HRT_EINVAL, "source fluxes not uploaded for every source and launched band");
    if ((uint64_t)ctx->n * (uint64_t)ctx->S >= 0xFFFFFFFFull)  // (primitive, source) sum keys are 32-bit
        return fail(ctx, HRT_EUNSUPPORTED, "primitives x sources of a direct pass must stay below 2^32");
    size_t ng = (size_t)ctx->n * ctx->S * 2;
    CU(ctx->Gd.ensure(ctx->stream, ng * sizeof(double)));
    CU(cudaMemsetAsync(ctx->Gd.p, 0, ng * sizeof(double), ctx->stream));
    DirectParams P;
    P.sc = scene_of(ctx);
    P.src = ctx->src.as<SourceDev>();
    P.S = ctx->S;
    P.dimx = dimx;
    P.dimy = dimy;
    P.seed = seed;
    P.pass = pass;
    P.offset = offset;
    P.count = count;
    P.G = ctx->Gd.as<double>();
    P.gl = GlassParams{};
    const uint32_t *cov = nullptr;
    int r;
    if ((r = covers_for(ctx, Bg, ctx->S, &cov))) return r;
    if (cov) {
        if (Bc > kGlassBands) return fail(ctx, HRT_EUNSUPPORTED, "at most 16 bands can be launched with translucent covers");
        const size_t nc = ng * (size_t)Bl;
        CU(ctx->Gcov.ensure(ctx->stream, nc * sizeof(double)));
        CU(cudaMemsetAsync(ctx->Gcov.p, 0, nc * sizeof(double), ctx->stream));
        P.sc.cover = cov;
        P.gl = glass_params(ctx, Bg, Bl);
        P.gl.Gcov = ctx->Gcov.as<double>();
        P.gl.src_flux = ctx->src_flux.as<float>();
    }
    if (ctx->measure & 4) P.sc.nodes4 = nullptr;  // counting on the binary tree, as the oracle does
    const uint32_t per = chunk_prims(ctx, (uint64_t)dimx * (uint64_t)dimy);
    if (per == 0) return HRT_EUNSUPPORTED;
    uint32_t chunks = 0;
    CU(timed_launch(ctx, 0, [&] {
        DirectParams Q = P;
        for (uint32_t done = 0; done < count; done += Q.count, ++chunks) {
            Q.offset = offset + done;
            Q.count = std::min(per, count - done);
            const cudaError_t e = cov ? launch_direct_glass(Q, max_blocks(ctx), ctx->stream)
                                      : ((ctx->measure & 1) ? launch_direct_stats(Q, max_blocks(ctx), ctx->stream)
                                                            : launch_direct(Q, max_blocks(ctx), ctx->stream));
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }));
    EpilogueParams E{};
    E.n = ctx->n;
    E.Bc = Bc;
    E.Bl = Bl;
    E.Bg = Bg;
    E.S = ctx->S;
    E.flags = ctx->flags.as<uint8_t>();
    E.rho = ctx->rho.as<float>();
    E.tau = ctx->tau.as<float>();
    E.rin = ctx->rin.as<double>();
    E.stop = ctx->stop.as<double>();
    E.sbot = ctx->sbot.as<double>();
    E.Gd = ctx->Gd.as<double>();
    E.Gcov = cov ? ctx->Gcov.as<double>() : nullptr;
    E.src_flux = ctx->src_flux.as<float>();
    CU(launch_epilogue_direct(E, ctx->stream));
    ctx->last_kernels += 1 + chunks;
    return HRT_OK;
}

// Diffuse pass over one or both faces + epilogue (__raygen__diffuse, __closesthit__diffuse, __miss__diffuse).
// ------------------------------------------------------------------ tuner --
// The diffuse trace has interchangeable kernel variants (persistent with 4 or 3 resident
// blocks per SM -- 64 registers with a few spills, or ~80 without -- and one ray per
// thread).  Which is fastest depends on the scene (BVH depth, primitive mix) and on the
// band count, so the first pass of each shape is timed on a sample: the rays of the
// first max(count/32, 4096) primitives, written to scratch sums (or the hit buffer of a
// recorded pass, rewritten by the real pass) and not counted.  The choice is cached
// per (mode, n, count, rays per face, faces, bands, voxels); passes under kTuneMinRays
// rays keep the default.  Choices differ only in the order of the FP64 atomic sums.
constexpr long long kTuneMinRays = 20000000;

const char *variant_name(int v) {
    switch (v) {
        case DV_W4: return "wide4";
        case DV_W43: return "wide4-3";
        case DV_W4S4: return "lean4";
        case DV_W4S5: return "lean5";
        case DV_W4S4D16: return "lean4-s16";
        case DV_W4B128: return "lean4-b128";
        case DV_W4B512: return "lean4-b512";
        case DV_W4K4: return "lean4-k4";
        case DV_W4K16: return "lean4-k16";
        case DV_W4S4D32: return "lean4-s32";
        case DV_PS4: return "binary4";
        case DV_PS3: return "binary3";
        case DV_SIMPLE: return "simple";
        default: return "default";
    }
}

int tuned_variant(hrt_context *ctx, const DiffuseParams &P0, bool record, int *variant) {
    const int nf = ((P0.faces & 1) ? 1 : 0) + ((P0.faces & 2) ? 1 : 0);
    const long long rays = (long long)P0.count * P0.dimx * P0.dimy * nf;
    *variant = record ? (P0.sc.nodes4 ? DV_W4 : DV_PS3) : DV_DEFAULT;
    if (ctx->tune >= 16) {  // forced variant (tests, experiments)
        const int v = ctx->tune - 16;
        if (!(record && v == DV_SIMPLE)) *variant = v;
        return HRT_OK;
    }
    if (!ctx->tune || rays < kTuneMinRays) return HRT_OK;
    char key[160];
    std::snprintf(key, sizeof key, "%s n=%d count=%u rays_per_face=%d faces=%d bands=%d voxels=%d",
                  record ? "record" : "accumulate", ctx->n, P0.count, P0.dimx * P0.dimy, P0.faces, P0.Bc,
                  P0.sc.voxels);
    auto it = ctx->tuned.find(key);
    if (it != ctx->tuned.end()) {
        *variant = it->second;
        return HRT_OK;
    }
    if (ctx->measure & 1) return HRT_OK;  // statistics launches count on a tuned choice, never time one
    std::vector<int> cand;
    const bool w4 = P0.sc.nodes4 != nullptr;
    if (record)
        cand = w4 ? std::vector<int>{DV_W4, DV_W43, DV_W4S4, DV_W4S5, DV_W4S4D16, DV_W4S4D32, DV_W4B128, DV_W4B512,
                                     DV_W4K4, DV_W4K16, DV_PS3, DV_PS4}
                  : std::vector<int>{DV_PS3, DV_PS4};
    else if (P0.sc.voxels) cand = w4 ? std::vector<int>{DV_W4, DV_PS4, DV_SIMPLE} : std::vector<int>{DV_PS4, DV_SIMPLE};
    else cand = w4 ? std::vector<int>{DV_W4, DV_W43, DV_W4S4, DV_W4S5, DV_W4S4D16, DV_W4S4D32, DV_W4B128, DV_W4B512,
                                      DV_W4K4, DV_W4K16, DV_PS4, DV_PS3, DV_SIMPLE}
                   : std::vector<int>{DV_PS4, DV_PS3, DV_SIMPLE};
    DiffuseParams P = P0;
    P.count = std::min(P0.count, std::max(P0.count / 32u, 4096u));
    // the sample is one launch: keep it within the per-launch ray limit
    P.count = std::min(P.count, std::max(launch_chunk_prims((uint64_t)P0.dimx * P0.dimy * nf, ctx->ray_limit), 1u));
    P.sc.rays = nullptr;
    P.sc.visits = nullptr;
    if (!record) {
        const size_t m = (size_t)ctx->n * P0.Bl;
        CU(ctx->tune_g.ensure(ctx->stream, 2 * m * sizeof(double)));
        P.Gt = ctx->tune_g.as<double>();
        P.Gb = P.Gt + m;
    }
    DiffuseParams W = P;  // warm-up launch (loads the kernel) on a smaller sample, same scratch outputs
    W.count = std::min(P.count, std::max(P.count / 8u, 1024u));
    cudaEvent_t a = nullptr, b = nullptr;
    CU(cudaEventCreate(&a));
    CU(cudaEventCreate(&b));
    auto launch_on = [&](const DiffuseParams &Q, int v) {
        return record ? launch_diffuse_record(Q, P0.hits, v, ctx->stream)
                      : launch_diffuse_variant(Q, v, max_blocks(ctx), ctx->stream);
    };
    auto launch = [&](int v) { return launch_on(P, v); };
    int best = cand[0];
    float best_ms = 1e30f;
    std::string line = std::string(key) + ":";
    cudaError_t e = cudaSuccess;
    for (int v : cand) {
        float ms = 0.f;
        if ((e = launch_on(W, v)) != cudaSuccess) break;  // loads the kernel
        if ((e = cudaEventRecord(a, ctx->stream)) != cudaSuccess || (e = launch(v)) != cudaSuccess ||
            (e = cudaEventRecord(b, ctx->stream)) != cudaSuccess || (e = cudaEventSynchronize(b)) != cudaSuccess ||
            (e = cudaEventElapsedTime(&ms, a, b)) != cudaSuccess)
            break;
        char t[48];
        std::snprintf(t, sizeof t, " %s=%.3fms", variant_name(v), ms);
        line += t;
        if (ms < best_ms) {
            best_ms = ms;
            best = v;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    CU(e);
    line += std::string(" -> ") + variant_name(best) + "\n";
    ctx->tune_log += line;
    ctx->tuned[key] = best;
    *variant = best;
    return HRT_OK;
}

int diffuse_pass(hrt_context *ctx, uint32_t offset, uint32_t count, uint32_t rpp, uint32_t seed, uint32_t pass, int faces,
                 int Bg, int Bc, int Bl, const SkyParams &sky) {
    int dimx, dimy;
    strata(rpp, &dimx, &dimy);
    if (dimx * dimy == 0 || count == 0 || Bc == 0) return HRT_OK;
    if (ctx->mS < 1 || ctx->mN != ctx->n)
        return fail(ctx, HRT_EINVAL, "materials do not match the geometry; call hrt_update_materials()");
    if (Bc > 16) return fail(ctx, HRT_EUNSUPPORTED, "at most 16 bands can be launched together");
    const int nfaces = ((faces & 1) ? 1 : 0) + ((faces & 2) ? 1 : 0);
    const uint32_t per = chunk_prims(ctx, (uint64_t)dimx * (uint64_t)dimy * (uint64_t)nfaces);
    if (per == 0) return HRT_EUNSUPPORTED;
    size_t m = (size_t)ctx->n * Bl;
    CU(cudaMemsetAsync(ctx->Gt.p, 0, m * sizeof(double), ctx->stream));
    CU(cudaMemsetAsync(ctx->Gb.p, 0, m * sizeof(double), ctx->stream));
    DiffuseParams P;
    P.sc = scene_of(ctx);
    P.dimx = dimx;
    P.dimy = dimy;
    P.seed = seed;
    P.pass = pass;
    P.offset = offset;
    P.count = count;
    P.faces = faces;
    P.Bc = Bc;
    P.Bl = Bl;
    P.otop = ctx->otop.as<float>();
    P.obot = ctx->obot.as<float>();
    P.sky = sky;
    P.Gt = ctx->Gt.as<double>();
    P.Gb = ctx->Gb.as<double>();
    CU(ctx->fetch.ensure(ctx->stream, sizeof(unsigned long long)));
    P.fetch = ctx->fetch.as<unsigned long long>();
    P.lane_budget = ctx->lane_budget;
    P.hits = nullptr;
    P.gl = GlassParams{};
    int variant = DV_DEFAULT, r;
    const uint32_t *cov = nullptr;
    if ((r = covers_for(ctx, Bg, 1, &cov))) return r;
    if (cov) {
        P.sc.cover = cov;
        P.gl = glass_params(ctx, Bg, Bl);
    } else if ((r = tuned_variant(ctx, P, false, &variant))) {
        return r;
    }
    uint32_t chunks = 0;
    CU(timed_launch(ctx, 1, [&] {
        DiffuseParams Q = P;
        for (uint32_t done = 0; done < count; done += Q.count, ++chunks) {
            Q.offset = offset + done;
            Q.count = std::min(per, count - done);
            const cudaError_t e =
                cov ? launch_diffuse_glass(Q, max_blocks(ctx), ctx->stream)
                    : ((ctx->measure & 1) ? launch_diffuse_stats(Q, (ctx->measure & 4) ? DV_SIMPLE : variant,
                                                                 max_blocks(ctx), ctx->stream)
                                          : launch_diffuse_variant(Q, variant, max_blocks(ctx), ctx->stream));
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }));
    EpilogueParams E{};
    E.n = ctx->n;
    E.Bc = Bc;
    E.Bl = Bl;
    E.Bg = Bg;
    E.S = 1;
    E.flags = ctx->flags.as<uint8_t>();
    E.rho = ctx->rho.as<float>();
    E.tau = ctx->tau.as<float>();
    E.rin = ctx->rin.as<double>();
    E.stop = ctx->stop.as<double>();
    E.sbot = ctx->sbot.as<double>();
    E.Gt = ctx->Gt.as<double>();
    E.Gb = ctx->Gb.as<double>();
    E.strength = 1.0 / (double)(dimx * dimy);
    CU(launch_epilogue_diffuse(E, ctx->stream));
    ctx->last_kernels += 1 + chunks;
    return HRT_OK;
}

// Camera parameters of a launch over the context's current radiation_out and sources.
int camera_params(hrt_context *ctx, const hrt_camera *c, int Bl, CameraParams *P) {
    if (!c) return fail(ctx, HRT_EINVAL, "null camera");
    const int W = c->resolution[0], H = c->resolution[1];
    const int tw = c->tile_resolution[0] > 0 ? c->tile_resolution[0] : W;
    const int th = c->tile_resolution[1] > 0 ? c->tile_resolution[1] : H;
    if (W <= 0 || H <= 0 || c->antialiasing < 1 || !(c->fov_aspect > 0.f) || !(c->viewplane_length > 0.f))
        return fail(ctx, HRT_EINVAL, "camera needs a resolution, >= 1 antialiasing sample, a field of view and an aspect ratio");
    if (c->tile_offset[0] < 0 || c->tile_offset[1] < 0 || c->tile_offset[0] + tw > W || c->tile_offset[1] + th > H)
        return fail(ctx, HRT_EINVAL, "camera tile lies outside the image");
    if ((long long)W * H > 0x7FFFFFFFLL || (long long)tw * th * c->antialiasing > 0xFFFFFFFFLL)
        return fail(ctx, HRT_EUNSUPPORTED, "camera image or tile too large for one launch");
    if (Bl <= 0 || Bl > 16) return fail(ctx, HRT_EINVAL, "a camera launch needs 1 to 16 bands in the radiation buffers");
    if (ctx->S > 0 && ctx->src_flux_count < (size_t)ctx->S * Bl)
        return fail(ctx, HRT_EINVAL, "source fluxes not uploaded for every source and launched band");
    CameraParams &q = *P;
    q = CameraParams{};
    q.sc = scene_of(ctx);
    for (int i = 0; i < 3; ++i) q.pos[i] = c->position[i];
    camera_rotation(c->direction[0], c->direction[1], q.M);
    q.focal = c->focal_length;
    q.lens = c->lens_diameter;
    q.inv_aspect = 1.0f / c->fov_aspect;
    q.viewplane = c->viewplane_length;
    q.W = W;
    q.H = H;
    q.ox = c->tile_offset[0];
    q.oy = c->tile_offset[1];
    q.tw = tw;
    q.th = th;
    q.aa = c->antialiasing;
    q.seed = c->seed;
    q.cam_id = c->camera_id;
    q.Bl = Bl;
    q.S = ctx->S;
    q.src = ctx->src.as<SourceDev>();
    q.src_flux = ctx->src_flux.as<float>();
    q.otop = ctx->otop.as<float>();
    q.obot = ctx->obot.as<float>();
    q.sky = SkyParams{};
    if (ctx->sky_B == Bl) {
        const size_t B = (size_t)Bl;
        float *d = ctx->cam_sky.as<float>();
        q.sky_rad = ctx->sky_has[0] ? d : nullptr;
        q.disk_rad = ctx->sky_has[1] ? d + B : nullptr;
        q.dflux = ctx->sky_has[2] ? d + 2 * B : nullptr;
        q.sky.prague = ctx->sky_has[3] ? d + 3 * B : nullptr;
        q.sky.peak = d + 7 * B;
        q.emission = ctx->sky_has[4] ? ctx->cam_em.as<uint32_t>() : nullptr;
        for (int i = 0; i < 3; ++i) q.sun[i] = ctx->sky_sun[i];
        q.disk_cos = ctx->sky_cos;
    }
    q.pix = ctx->cam_pix.as<double>();
    q.labels = ctx->cam_lab.as<uint32_t>();
    q.depths = ctx->cam_dep.as<float>();
    return HRT_OK;
}

int ensure_camera_image(hrt_context *ctx, int W, int H, int Bl) {
    const size_t npx = (size_t)W * H;
    CU(ctx->cam_pix.ensure(ctx->stream, npx * Bl * sizeof(double)));
    CU(cudaMemsetAsync(ctx->cam_pix.p, 0, npx * Bl * sizeof(double), ctx->stream));
    ctx->cam_W = W;
    ctx->cam_H = H;
    ctx->cam_B = Bl;
    return HRT_OK;
}

int ensure_camera_labels(hrt_context *ctx, int W, int H) {
    const size_t npx = (size_t)W * H;
    CU(ctx->cam_lab.ensure(ctx->stream, npx * sizeof(uint32_t)));
    CU(ctx->cam_dep.ensure(ctx->stream, npx * sizeof(float)));
    CU(cudaMemsetAsync(ctx->cam_lab.p, 0, npx * sizeof(uint32_t), ctx->stream));
    CU(cudaMemsetAsync(ctx->cam_dep.p, 0, npx * sizeof(float), ctx->stream));
    ctx->lab_W = W;
    ctx->lab_H = H;
    return HRT_OK;
}

// Energy balance: upload the surface arrays of n primitives.
int upload_surface(hrt_context *ctx, int n, const hrt_surface *s) {
    if (!s) return fail(ctx, HRT_EINVAL, "null surface");
    const float *a[10] = {s->air_temperature, s->air_vapor_pressure, s->air_pressure, s->bl_conductance,
                          s->moisture_conductance, s->emissivity, s->other_flux, s->heat_capacity,
                          s->surface_humidity, s->stomatal_sidedness};
    for (const float *x : a)
        if (!x) return fail(ctx, HRT_EINVAL, "null surface array");
    if (!s->nsides) return fail(ctx, HRT_EINVAL, "null surface array");
    if (!(s->dt >= 0.f)) return fail(ctx, HRT_EINVAL, "dt must be >= 0");
    const size_t N = (size_t)n;
    CU(ctx->eb_surf.ensure(ctx->stream, 10 * N * sizeof(float)));
    CU(ctx->eb_sides.ensure(ctx->stream, N));
    for (int k = 0; k < 10; ++k)
        CU(cudaMemcpyAsync(ctx->eb_surf.as<float>() + k * N, a[k], N * sizeof(float), cudaMemcpyHostToDevice,
                           ctx->stream));
    CU(cudaMemcpyAsync(ctx->eb_sides.p, s->nsides, N, cudaMemcpyHostToDevice, ctx->stream));
    CU(ctx->eb_R.ensure(ctx->stream, N * sizeof(float)));
    CU(ctx->eb_T.ensure(ctx->stream, N * sizeof(float)));
    CU(ctx->eb_out.ensure(ctx->stream, 5 * N * sizeof(float)));
    CU(ctx->eb_status.ensure(ctx->stream, 2 * sizeof(unsigned)));
    ctx->eb_n = n;
    ctx->eb_dt = s->dt;
    ctx->eb_Tdef = s->temperature_default;
    return HRT_OK;
}

// One energy-balance solve over the uploaded surface: R (device [n]) and Tin (device [n]) to
// ctx->eb_T; counts unconverged primitives into eb_status[0].
int eb_solve(hrt_context *ctx, const float *R, const float *Tin, bool outputs) {
    const size_t N = (size_t)ctx->eb_n;
    EnergyParams P{};
    P.n = ctx->eb_n;
    P.R = R;
    P.Tin = Tin;
    const float *f = ctx->eb_surf.as<float>();
    P.Ta = f;
    P.ea = f + N;
    P.press = f + 2 * N;
    P.gH = f + 3 * N;
    P.gS = f + 4 * N;
    P.eps = f + 5 * N;
    P.Qother = f + 6 * N;
    P.cap = f + 7 * N;
    P.hs = f + 8 * N;
    P.sided = f + 9 * N;
    P.nsides = ctx->eb_sides.as<uint8_t>();
    P.dt = ctx->eb_dt;
    P.T_default = ctx->eb_Tdef;
    P.Tout = ctx->eb_T.as<float>();
    P.out = outputs ? ctx->eb_out.as<float>() : nullptr;
    P.status = ctx->eb_status.as<unsigned>();
    CU(cudaMemsetAsync(ctx->eb_status.p, 0, 2 * sizeof(unsigned), ctx->stream));
    CU(launch_energy_balance(P, ctx->stream));
    return HRT_OK;
}

int count_flags(int Bg, const uint8_t *f) {
    int c = 0;
    for (int b = 0; b < Bg; ++b) c += f[b] ? 1 : 0;
    return c;
}

}  // namespace

// ============================================================== C ABI ===
extern "C" {

const char *hrt_backend_name(void) { return "GB300 sm_103a (hrt)"; }

int hrt_create(hrt_context **out, int device) {
    if (!out) return HRT_EINVAL;
    *out = nullptr;
    hrt_context *ctx = new hrt_context();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        delete ctx;
        return HRT_ECUDA;
    }
    cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return HRT_ECUDA;
    }
    ctx->stream = ctx->own;
    keep_pool(device);
    if (ctx->status.ensure(ctx->stream, sizeof(uint32_t)) != cudaSuccess || ctx->counter.ensure(ctx->stream, sizeof(unsigned long long)) != cudaSuccess) {
        cudaStreamDestroy(ctx->own);
        delete ctx;
        return HRT_ENOMEM;
    }
    cudaMemsetAsync(ctx->status.p, 0, sizeof(uint32_t), ctx->stream);
    cudaMemsetAsync(ctx->counter.p, 0, sizeof(unsigned long long), ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        cudaStreamDestroy(ctx->own);
        delete ctx;
        return HRT_ECUDA;
    }
    *out = ctx;
    return HRT_OK;
}

int hrt_destroy(hrt_context *ctx) {
    if (!ctx) return HRT_EINVAL;
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream, own = ctx->own;
    cudaStreamSynchronize(s);
    if (ctx->sw_exec) cudaGraphExecDestroy(ctx->sw_exec);
    if (ctx->mw_exec) cudaGraphExecDestroy(ctx->mw_exec);
    collect_timings(ctx);
    g_release_stream = s;  // buffers are released on the context's stream
    delete ctx;
    g_release_stream = nullptr;
    cudaStreamSynchronize(s);
    if (own) cudaStreamDestroy(own);
    return HRT_OK;
}

const char *hrt_last_error(const hrt_context *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int hrt_set_stream(hrt_context *ctx, void *stream) {
    if (!ctx) return HRT_EINVAL;
    CU(cudaSetDevice(ctx->device));
    CU(cudaStreamSynchronize(ctx->stream));  // buffers allocated on the old stream are ready
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
    return HRT_OK;
}

int hrt_update_geometry(hrt_context *ctx, const hrt_geometry *g) {
    if (!ctx || !g) return HRT_EINVAL;
    if (g->n < 0) return fail(ctx, HRT_EINVAL, "negative primitive count");
    if (g->n > 0 && (!g->transform || !g->type || !g->twosided))
        return fail(ctx, HRT_EINVAL, "null geometry array");
    if (!(g->nbbox == 0 || g->nbbox == 2 || g->nbbox == 4) || (g->nbbox > 0 && !g->bbox_vertices))
        return fail(ctx, HRT_EINVAL, "periodic walls must be 0, 2 or 4 quads");
    ctx->cover_key.clear();
    std::vector<uint32_t> voxels;
    for (int i = 0; i < g->n; ++i) {
        if (g->type[i] > 4) return fail(ctx, HRT_EUNSUPPORTED, "unsupported primitive type " + std::to_string(g->type[i]));
        if (g->type[i] == PT_VOXEL) voxels.push_back((uint32_t)i);
    }
    if (!voxels.empty()) {
        if (!g->voxel_lad) return fail(ctx, HRT_EINVAL, "voxels need voxel_lad (leaf area density)");
        for (uint32_t i : voxels)
            if (!(g->voxel_lad[i] >= 0.f) || std::isinf(g->voxel_lad[i]))
                return fail(ctx, HRT_EINVAL, "voxel leaf area density must be finite and >= 0");
    }
    CU(cudaSetDevice(ctx->device));
    size_t n = (size_t)g->n;
    CU(ctx->T.ensure(ctx->stream, std::max<size_t>(n, 1) * 16 * sizeof(float)));
    CU(ctx->type.ensure(ctx->stream, std::max<size_t>(n, 1) * sizeof(uint32_t)));
    CU(ctx->twosided.ensure(ctx->stream, std::max<size_t>(n, 1)));
    CU(ctx->area.ensure(ctx->stream, std::max<size_t>(n, 1) * sizeof(double)));
    ctx->h_twosided.assign(g->twosided, g->twosided + n);
    for (uint32_t i : voxels) ctx->h_twosided[i] = 1;  // a voxel launches both directions of each sample
    // primitive areas (voxels: leaf area) weight the scattering residual
    std::vector<double> area(n);
    for (size_t i = 0; i < n; ++i)
        area[i] = prim_area(g->transform + 16 * i, g->type[i], g->type[i] == PT_VOXEL ? g->voxel_lad[i] : 0.f);
    if (n) {
        CU(cudaMemcpyAsync(ctx->T.p, g->transform, n * 16 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        CU(cudaMemcpyAsync(ctx->type.p, g->type, n * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
        CU(cudaMemcpyAsync(ctx->twosided.p, ctx->h_twosided.data(), n, cudaMemcpyHostToDevice, ctx->stream));
        CU(cudaMemcpyAsync(ctx->area.p, area.data(), n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    }
    if (!voxels.empty()) {
        CU(ctx->lad.ensure(ctx->stream, n * sizeof(float)));
        CU(cudaMemcpyAsync(ctx->lad.p, g->voxel_lad, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    }
    ctx->h_voxels.swap(voxels);
    // texture masks
    ctx->masks = false;
    if (g->mask_id && g->nmasks > 0 && n) {
        if (!g->mask_size || !g->mask_data) return fail(ctx, HRT_EINVAL, "masks need mask_size and mask_data");
        std::vector<uint32_t> off((size_t)g->nmasks);
        size_t total = 0;
        for (int k = 0; k < g->nmasks; ++k) {
            if (g->mask_size[2 * k] < 1 || g->mask_size[2 * k + 1] < 1) return fail(ctx, HRT_EINVAL, "empty mask");
            off[k] = (uint32_t)total;
            total += (size_t)g->mask_size[2 * k] * (size_t)g->mask_size[2 * k + 1];
        }
        if (total >= (1ull << 32)) return fail(ctx, HRT_EINVAL, "mask data above 4 GB");
        for (size_t i = 0; i < n; ++i)
            if (g->mask_id[i] >= g->nmasks || g->mask_id[i] < -1) return fail(ctx, HRT_EINVAL, "mask id out of range");
        std::vector<int32_t> uvid(n, -1);
        std::vector<float> uv(8 * n, 0.f);
        if (g->uv_id && g->uv) {
            uvid.assign(g->uv_id, g->uv_id + n);
            uv.assign(g->uv, g->uv + 8 * n);
        }
        CU(ctx->mask_id.ensure(ctx->stream, n * sizeof(int32_t)));
        CU(ctx->mask_uv_id.ensure(ctx->stream, n * sizeof(int32_t)));
        CU(ctx->mask_uv.ensure(ctx->stream, 8 * n * sizeof(float)));
        CU(ctx->mask_size.ensure(ctx->stream, 2 * (size_t)g->nmasks * sizeof(int32_t)));
        CU(ctx->mask_offset.ensure(ctx->stream, (size_t)g->nmasks * sizeof(uint32_t)));
        CU(ctx->mask_data.ensure(ctx->stream, std::max<size_t>(total, 1)));
        CU(cudaMemcpyAsync(ctx->mask_id.p, g->mask_id, n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
        CU(cudaMemcpyAsync(ctx->mask_uv_id.p, uvid.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
        CU(cudaMemcpyAsync(ctx->mask_uv.p, uv.data(), 8 * n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        CU(cudaMemcpyAsync(ctx->mask_size.p, g->mask_size, 2 * (size_t)g->nmasks * sizeof(int32_t),
                           cudaMemcpyHostToDevice, ctx->stream));
        CU(cudaMemcpyAsync(ctx->mask_offset.p, off.data(), off.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                           ctx->stream));
        CU(cudaMemcpyAsync(ctx->mask_data.p, g->mask_data, total, cudaMemcpyHostToDevice, ctx->stream));
        ctx->masks = true;
    }
    ctx->nbbox = g->nbbox;
    ctx->px = g->periodic_x;
    ctx->py = g->periodic_y;
    if (g->nbbox) {
        std::vector<float4> q((size_t)g->nbbox * 4);
        for (int i = 0; i < g->nbbox * 4; ++i)
            q[i] = make_float4(g->bbox_vertices[3 * i], g->bbox_vertices[3 * i + 1], g->bbox_vertices[3 * i + 2], 0.f);
        CU(ctx->bbox.ensure(ctx->stream, q.size() * sizeof(float4)));
        CU(cudaMemcpyAsync(ctx->bbox.p, q.data(), q.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
    }
    ctx->n = g->n;
    ctx->have_geometry = true;
    ctx->built = false;
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_build_accel(hrt_context *ctx) {
    if (!ctx) return HRT_EINVAL;
    if (!ctx->have_geometry) return fail(ctx, HRT_EINVAL, "hrt_update_geometry() has not been called");
    CU(cudaSetDevice(ctx->device));
    int n = ctx->n;
    if (n == 0) {
        ctx->built = true;
        return HRT_OK;
    }
    size_t nn = (size_t)n, ni = (size_t)std::max(n - 1, 1);
    CU(ctx->rec.ensure(ctx->stream, nn * 4 * sizeof(float4)));
    CU(ctx->rgen.ensure(ctx->stream, nn * 4 * sizeof(float4)));
    CU(ctx->nodes.ensure(ctx->stream, ni * 4 * sizeof(float4)));
    CU(ctx->codes.ensure(ctx->stream, nn * sizeof(uint64_t)));
    CU(ctx->perm.ensure(ctx->stream, nn * sizeof(uint32_t)));
    CU(ctx->bvh_scratch.ensure(ctx->stream, bvh_scratch_bytes(n)));
    BvhBuffers b;
    bvh_carve(b, ctx->bvh_scratch.p, n);
    b.rec = ctx->rec.as<float4>();
    b.rgen = ctx->rgen.as<float4>();
    b.nodes = ctx->nodes.as<float4>();
    b.codes = ctx->codes.as<uint64_t>();
    b.perm = ctx->perm.as<uint32_t>();
    b.status = ctx->status.as<uint32_t>();
    CU(bvh_build(ctx->T.as<float>(), ctx->type.as<uint32_t>(), ctx->h_voxels.empty() ? nullptr : ctx->lad.as<float>(), n,
                 b, ctx->stream));
    int r = sync_and_status(ctx);
    if (r) return r;
    // compressed 4-wide nodes for the persistent diffuse trace (scratch reuses the build's)
    ctx->n4 = 0;
    CU(ctx->nodes4.ensure(ctx->stream, bvh4_node_capacity(n) * 4 * sizeof(float4)));
    // the traces fetch a node in two 256-bit loads, which need 32-byte aligned addresses
    if (((uintptr_t)ctx->nodes.p | (uintptr_t)ctx->nodes4.p) & 63u)
        return fail(ctx, HRT_ECUDA, "node arrays are not 64-byte aligned");
    if (bvh4_scratch_bytes(n) > ctx->bvh_scratch.cap) CU(ctx->bvh_scratch.ensure(ctx->stream, bvh4_scratch_bytes(n)));
    int n4 = 0;
    // the 4-wide nodes come from the clustered binary tree (fewer node visits than the
    // Morton split); its nodes and scratch live only for the build
    const float4 *src2 = ctx->nodes.as<float4>();
    DevBuf ploc_nodes, ploc_scratch;
    if (n >= 2) {
        CU(ploc_nodes.ensure(ctx->stream, ni * 4 * sizeof(float4)));
        CU(ploc_scratch.ensure(ctx->stream, ploc_scratch_bytes(n)));
        CU(ploc_build(b.leafbox, n, ploc_nodes.as<float4>(), ploc_scratch.p, ctx->stream));
        src2 = ploc_nodes.as<float4>();
    }
    CU(bvh4_build(src2, n, ctx->nodes4.as<float4>(), ctx->bvh_scratch.p, ctx->status.as<uint32_t>(), &n4,
                  ctx->stream));
    ploc_nodes.free_on(ctx->stream);
    ploc_scratch.free_on(ctx->stream);
    if ((r = sync_and_status(ctx))) return r;
    ctx->n4 = n4;
    ctx->built = true;
    return HRT_OK;
}

int hrt_update_materials(hrt_context *ctx, int32_t nsources, int32_t nprims, int32_t nbands_global, const float *rho,
                         const float *tau) {
    if (!ctx || nsources < 0 || nprims < 0 || nbands_global < 0) return HRT_EINVAL;
    size_t m = (size_t)nsources * nprims * nbands_global;
    if (m && (!rho || !tau)) return fail(ctx, HRT_EINVAL, "null material array");
    CU(cudaSetDevice(ctx->device));
    CU(ctx->rho.ensure(ctx->stream, std::max<size_t>(m, 1) * sizeof(float)));
    CU(ctx->tau.ensure(ctx->stream, std::max<size_t>(m, 1) * sizeof(float)));
    std::vector<float> vr, vt;
    if (m && !ctx->h_voxels.empty() && nprims == ctx->n) {
        // A voxel's leaves scatter rho + tau into one isotropic field: half of it is routed
        // to each face, so both faces emit the same radiance.
        vr.assign(rho, rho + m);
        vt.assign(tau, tau + m);
        for (int32_t src = 0; src < nsources; ++src)
            for (uint32_t p : ctx->h_voxels)
                for (int32_t b = 0; b < nbands_global; ++b) {
                    size_t i = ((size_t)src * nprims + p) * nbands_global + b;
                    float h = 0.5f * (vr[i] + vt[i]);
                    vr[i] = h;
                    vt[i] = h;
                }
        rho = vr.data();
        tau = vt.data();
    }
    if (m) {
        CU(cudaMemcpyAsync(ctx->rho.p, rho, m * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        CU(cudaMemcpyAsync(ctx->tau.p, tau, m * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    }
    ctx->mS = nsources;
    ctx->mN = nprims;
    ctx->mB = nbands_global;
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_update_glass(hrt_context *ctx, int32_t nsources, int32_t nprims, int32_t nbands_global, const int8_t *is_glass,
                     const float *glass_n, const float *glass_kl) {
    if (!ctx || nsources < 0 || nprims < 0 || nbands_global < 0) return HRT_EINVAL;
    CU(cudaSetDevice(ctx->device));
    ctx->cover_key.clear();
    const size_t m = (size_t)nsources * nprims * nbands_global;
    bool any = false;
    for (size_t i = 0; is_glass && i < m && !any; ++i) any = is_glass[i] != 0;
    if (!any) {
        ctx->gS = 0;
        ctx->h_glass.clear();
        return HRT_OK;
    }
    if (!glass_n || !glass_kl) return fail(ctx, HRT_EINVAL, "null translucent-cover array");
    if (nprims != ctx->n) return fail(ctx, HRT_EINVAL, "translucent-cover arrays do not match the geometry");
    if (nsources > 32) return fail(ctx, HRT_EUNSUPPORTED, "translucent covers take at most 32 sources");
    for (size_t i = 0; i < m; ++i) {
        if (!is_glass[i]) continue;
        if (!(glass_n[i] >= 1.f) || std::isinf(glass_n[i]) || !(glass_kl[i] >= 0.f) || std::isinf(glass_kl[i]))
            return fail(ctx, HRT_EINVAL, "a translucent cover needs a refractive index >= 1 and K*L >= 0");
    }
    CU(ctx->gn.ensure(ctx->stream, m * sizeof(float)));
    CU(ctx->gkl.ensure(ctx->stream, m * sizeof(float)));
    CU(cudaMemcpyAsync(ctx->gn.p, glass_n, m * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaMemcpyAsync(ctx->gkl.p, glass_kl, m * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    ctx->h_glass.assign(is_glass, is_glass + m);
    ctx->gS = nsources;
    ctx->gB = nbands_global;
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_update_sources(hrt_context *ctx, int32_t nsources, const hrt_source *sources) {
    if (!ctx || nsources < 0 || (nsources > 0 && !sources)) return HRT_EINVAL;
    if (nsources > 256) return fail(ctx, HRT_EINVAL, "A maximum of 256 radiation sources are allowed.");
    CU(cudaSetDevice(ctx->device));
    std::vector<SourceDev> h((size_t)std::max(nsources, 1));
    for (int k = 0; k < nsources; ++k) {
        if (sources[k].type > 4) return fail(ctx, HRT_EINVAL, "unknown source type");
        SourceDev &s = h[k];
        s.type = (int)sources[k].type;
        for (int i = 0; i < 3; ++i) s.pos[i] = sources[k].position[i];
        s.w0 = sources[k].width[0];
        s.w1 = sources[k].width[1];
        rotation3(sources[k].rotation, s.R);
    }
    CU(ctx->src.ensure(ctx->stream, h.size() * sizeof(SourceDev)));
    CU(cudaMemcpyAsync(ctx->src.p, h.data(), h.size() * sizeof(SourceDev), cudaMemcpyHostToDevice, ctx->stream));
    ctx->S = nsources;
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_upload_source_fluxes(hrt_context *ctx, const float *fluxes, size_t count) {
    if (!ctx || (count && !fluxes)) return HRT_EINVAL;
    CU(cudaSetDevice(ctx->device));
    CU(ctx->src_flux.ensure(ctx->stream, std::max<size_t>(count, 1) * sizeof(float)));
    if (count) CU(cudaMemcpyAsync(ctx->src_flux.p, fluxes, count * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    ctx->src_flux_count = count;
    ctx->h_src_flux.assign(fluxes, fluxes + count);
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_zero_radiation_buffers(hrt_context *ctx, size_t launch_band_count) {
    if (!ctx) return HRT_EINVAL;
    if (ctx->n == 0 || launch_band_count == 0) return HRT_OK;
    if ((int)launch_band_count > ctx->mB)
        return fail(ctx, HRT_EINVAL, "launch_band_count exceeds the band count of the materials; call hrt_update_materials() first");
    CU(cudaSetDevice(ctx->device));
    int r = ensure_buffers(ctx, (int)launch_band_count);
    if (r) return r;
    size_t m = (size_t)ctx->n * launch_band_count;
    CU(cudaMemsetAsync(ctx->rin.p, 0, m * sizeof(double), ctx->stream));
    CU(cudaMemsetAsync(ctx->stop.p, 0, m * sizeof(double), ctx->stream));
    CU(cudaMemsetAsync(ctx->sbot.p, 0, m * sizeof(double), ctx->stream));
    CU(cudaMemsetAsync(ctx->otop.p, 0, m * sizeof(float), ctx->stream));
    CU(cudaMemsetAsync(ctx->obot.p, 0, m * sizeof(float), ctx->stream));
    ctx->Bl = (int)launch_band_count;
    ctx->cam_id_cur = 0xFFFFFFFFu;  // the next camera launch starts a fresh image
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_zero_scatter_buffers(hrt_context *ctx) {
    if (!ctx) return HRT_EINVAL;
    if (ctx->n == 0 || ctx->Bl == 0) return HRT_OK;
    size_t m = (size_t)ctx->n * ctx->Bl;
    CU(cudaMemsetAsync(ctx->stop.p, 0, m * sizeof(double), ctx->stream));
    CU(cudaMemsetAsync(ctx->sbot.p, 0, m * sizeof(double), ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_copy_scatter_to_radiation(hrt_context *ctx) {
    if (!ctx) return HRT_EINVAL;
    if (ctx->n == 0 || ctx->Bl == 0) return HRT_OK;
    size_t m = (size_t)ctx->n * ctx->Bl;
    CU(launch_to_float(ctx->stop.as<double>(), ctx->otop.as<float>(), m, ctx->stream));
    CU(launch_to_float(ctx->sbot.as<double>(), ctx->obot.as<float>(), m, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_upload_radiation_out(hrt_context *ctx, const float *top, const float *bottom, size_t count) {
    if (!ctx) return HRT_EINVAL;
    size_t m = (size_t)ctx->n * ctx->Bl;
    if (count > m) return fail(ctx, HRT_EINVAL, "radiation_out larger than Nprims x Nbands_launch");
    if (top && count) CU(cudaMemcpyAsync(ctx->otop.p, top, count * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    if (bottom && count) CU(cudaMemcpyAsync(ctx->obot.p, bottom, count * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_get_results(hrt_context *ctx, float *radiation_in, float *out_top, float *out_bottom, float *scatter_top,
                    float *scatter_bottom) {
    if (!ctx) return HRT_EINVAL;
    size_t m = (size_t)ctx->n * ctx->Bl;
    if (m == 0) return HRT_OK;
    auto dl_double = [&](DevBuf &src, float *dst) -> int {
        if (!dst) return HRT_OK;
        CU(launch_to_float(src.as<double>(), ctx->fin.as<float>(), m, ctx->stream));
        CU(cudaMemcpyAsync(dst, ctx->fin.p, m * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
        return HRT_OK;
    };
    int r;
    if ((r = dl_double(ctx->rin, radiation_in))) return r;
    if ((r = dl_double(ctx->stop, scatter_top))) return r;
    if ((r = dl_double(ctx->sbot, scatter_bottom))) return r;
    if (out_top) CU(cudaMemcpyAsync(out_top, ctx->otop.p, m * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    if (out_bottom) CU(cudaMemcpyAsync(out_bottom, ctx->obot.p, m * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_energy_balance(hrt_context *ctx, int32_t n, const hrt_surface *s, const float *net_radiation,
                       const float *temperature, float *temperature_out, float *fluxes_out) {
    if (!ctx || n < 0) return HRT_EINVAL;
    if (n == 0) return HRT_OK;
    CU(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    int r = upload_surface(ctx, n, s);
    if (r) return r;
    const size_t N = (size_t)n;
    if (net_radiation) {
        CU(cudaMemcpyAsync(ctx->eb_R.p, net_radiation, N * sizeof(float), cudaMemcpyHostToDevice, st));
    } else {
        if (n != ctx->n || ctx->Bl <= 0 || !ctx->fin.p)
            return fail(ctx, HRT_EINVAL, "no device fluxes of this scene; call hrt_run_band() first or pass net_radiation");
        CU(launch_net_radiation(n, ctx->Bl, ctx->fin.as<float>(), ctx->eb_R.as<float>(), st));
    }
    if (temperature) {
        CU(ctx->emis_T.ensure(st, N * sizeof(float)));
        CU(cudaMemcpyAsync(ctx->emis_T.p, temperature, N * sizeof(float), cudaMemcpyHostToDevice, st));
        ctx->emis_T_count = N;
    } else if (ctx->emis_T_count != N) {
        return fail(ctx, HRT_EINVAL, "no resident temperatures for these primitives; pass temperature");
    }
    if ((r = eb_solve(ctx, ctx->eb_R.as<float>(), ctx->emis_T.as<float>(), fluxes_out != nullptr))) return r;
    CU(cudaMemcpyAsync(ctx->emis_T.p, ctx->eb_T.p, N * sizeof(float), cudaMemcpyDeviceToDevice, st));
    unsigned bad = 0;
    CU(cudaMemcpyAsync(&bad, ctx->eb_status.p, sizeof bad, cudaMemcpyDeviceToHost, st));
    if (temperature_out) CU(cudaMemcpyAsync(temperature_out, ctx->eb_T.p, N * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (fluxes_out) CU(cudaMemcpyAsync(fluxes_out, ctx->eb_out.p, 5 * N * sizeof(float), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    ctx->eb_unconverged = bad;
    return HRT_OK;
}

int hrt_run_coupled(hrt_context *ctx, const hrt_band_solve *s, const hrt_surface *surface, int32_t max_iterations,
                    float tolerance_K, float *flux_out, float *temperature_out, int32_t *iterations_out) {
    if (!ctx || !s || max_iterations < 1 || !(tolerance_K >= 0.f)) return HRT_EINVAL;
    int r = check_built(ctx);
    if (r) return r;
    CU(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int n = ctx->n;
    const size_t N = (size_t)n;
    if ((r = upload_surface(ctx, n, surface))) return r;
    hrt_band_solve later = *s;
    later.temperature = nullptr;
    later.emissivity = nullptr;
    later.rho = nullptr;
    later.tau = nullptr;
    later.sources = nullptr;
    later.source_flux = nullptr;
    later.ncameras = 0;
    int it = 0;
    uint64_t bad_total = 0;
    for (; it < max_iterations;) {
        if ((r = hrt_run_band(ctx, it == 0 ? s : &later, nullptr))) return r;
        if (ctx->emis_T_count != N)
            return fail(ctx, HRT_EINVAL, "the coupled solve needs temperatures (hrt_band_solve.temperature)");
        CU(launch_net_radiation(n, ctx->Bl, ctx->fin.as<float>(), ctx->eb_R.as<float>(), st));
        if ((r = eb_solve(ctx, ctx->eb_R.as<float>(), ctx->emis_T.as<float>(), false))) return r;
        CU(launch_max_abs_diff(n, ctx->eb_T.as<float>(), ctx->emis_T.as<float>(), ctx->eb_status.as<unsigned>() + 1, st));
        CU(cudaMemcpyAsync(ctx->emis_T.p, ctx->eb_T.p, N * sizeof(float), cudaMemcpyDeviceToDevice, st));
        unsigned h[2] = {0, 0};
        CU(cudaMemcpyAsync(h, ctx->eb_status.p, sizeof h, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        ++it;
        bad_total = h[0];
        float dmax;
        std::memcpy(&dmax, &h[1], sizeof dmax);
        if (dmax <= tolerance_K) break;
    }
    ctx->eb_unconverged = bad_total;
    const size_t m = N * (size_t)ctx->Bl;
    if (flux_out) CU(cudaMemcpyAsync(flux_out, ctx->fin.p, m * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (temperature_out) CU(cudaMemcpyAsync(temperature_out, ctx->emis_T.p, N * sizeof(float), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (iterations_out) *iterations_out = it;
    return HRT_OK;
}

int hrt_update_sky_model(hrt_context *ctx, int32_t nbands, const hrt_sky_model *m) {
    if (!ctx || nbands < 0) return HRT_EINVAL;
    CU(cudaSetDevice(ctx->device));
    if (!m || nbands == 0) {
        ctx->sky_B = 0;
        return HRT_OK;
    }
    const size_t B = (size_t)nbands;
    std::vector<float> h(10 * B, 0.f);
    const float *arr[3] = {m->camera_sky_radiance, m->solar_disk_radiance, m->camera_diffuse_flux};
    for (int k = 0; k < 3; ++k) {
        ctx->sky_has[k] = arr[k] != nullptr;
        if (arr[k]) std::copy(arr[k], arr[k] + B, h.begin() + k * B);
    }
    ctx->sky_has[3] = m->sky_radiance_params != nullptr;
    if (m->sky_radiance_params) std::copy(m->sky_radiance_params, m->sky_radiance_params + 4 * B, h.begin() + 3 * B);
    for (size_t b = 0; b < B; ++b)
        for (int i = 0; i < 3; ++i) h[7 * B + 3 * b + i] = m->sun_direction[i];
    CU(ctx->cam_sky.ensure(ctx->stream, h.size() * sizeof(float)));
    CU(cudaMemcpyAsync(ctx->cam_sky.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    ctx->sky_has[4] = m->band_emission_flag != nullptr;
    if (m->band_emission_flag) {
        CU(ctx->cam_em.ensure(ctx->stream, B * sizeof(uint32_t)));
        CU(cudaMemcpyAsync(ctx->cam_em.p, m->band_emission_flag, B * sizeof(uint32_t), cudaMemcpyHostToDevice,
                           ctx->stream));
    }
    for (int i = 0; i < 3; ++i) ctx->sky_sun[i] = m->sun_direction[i];
    ctx->sky_cos = m->solar_disk_cos_angle;
    ctx->sky_B = nbands;
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_launch_camera(hrt_context *ctx, const hrt_camera *cam) {
    if (!ctx || !cam) return HRT_EINVAL;
    int r = check_built(ctx);
    if (r) return r;
    CU(cudaSetDevice(ctx->device));
    CameraParams P;
    if ((r = camera_params(ctx, cam, ctx->Bl, &P))) return r;
    if (cam->camera_id != ctx->cam_id_cur || ctx->Bl != ctx->cam_B || P.W != ctx->cam_W || P.H != ctx->cam_H) {
        if ((r = ensure_camera_image(ctx, P.W, P.H, ctx->Bl))) return r;
        ctx->cam_id_cur = cam->camera_id;
        P.pix = ctx->cam_pix.as<double>();
    }
    CU(cudaMemsetAsync(ctx->counter.p, 0, sizeof(unsigned long long), ctx->stream));
    CU(launch_camera(P, max_blocks(ctx), ctx->stream));
    return sync_and_status(ctx);
}

int hrt_zero_camera_pixel_buffers(hrt_context *ctx, int32_t width, int32_t height) {
    if (!ctx || width < 0 || height < 0) return HRT_EINVAL;
    if ((size_t)width * height == 0) return HRT_OK;
    CU(cudaSetDevice(ctx->device));
    int r = ensure_camera_labels(ctx, width, height);
    if (r) return r;
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_launch_pixel_labels(hrt_context *ctx, const hrt_camera *cam) {
    if (!ctx || !cam) return HRT_EINVAL;
    int r = check_built(ctx);
    if (r) return r;
    CU(cudaSetDevice(ctx->device));
    CameraParams P;
    if ((r = camera_params(ctx, cam, std::max(ctx->Bl, 1), &P))) return r;
    if (P.W != ctx->lab_W || P.H != ctx->lab_H) {
        if ((r = ensure_camera_labels(ctx, P.W, P.H))) return r;
        P.labels = ctx->cam_lab.as<uint32_t>();
        P.depths = ctx->cam_dep.as<float>();
    }
    CU(launch_pixel_labels(P, ctx->stream));
    return sync_and_status(ctx);
}

int hrt_get_camera_results(hrt_context *ctx, float *pixels, uint32_t *labels, float *depths, int32_t width,
                           int32_t height) {
    if (!ctx || width < 0 || height < 0) return HRT_EINVAL;
    CU(cudaSetDevice(ctx->device));
    const size_t npx = (size_t)width * height;
    if (npx == 0) return HRT_OK;
    if (pixels) {
        if (ctx->cam_W != width || ctx->cam_H != height)
            return fail(ctx, HRT_EINVAL, "no camera image of this resolution; call hrt_launch_camera() first");
        const size_t m = npx * ctx->cam_B;
        CU(ctx->io_a.ensure(ctx->stream, m * sizeof(float)));
        CU(launch_to_float(ctx->cam_pix.as<double>(), ctx->io_a.as<float>(), m, ctx->stream));
        CU(cudaMemcpyAsync(pixels, ctx->io_a.p, m * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (labels || depths) {
        if (ctx->lab_W != width || ctx->lab_H != height)
            return fail(ctx, HRT_EINVAL, "no pixel labels of this resolution; call hrt_launch_pixel_labels() first");
        if (labels) CU(cudaMemcpyAsync(labels, ctx->cam_lab.p, npx * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
        if (depths) CU(cudaMemcpyAsync(depths, ctx->cam_dep.p, npx * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CU(cudaStreamSynchronize(ctx->stream));
    return HRT_OK;
}

int hrt_launch_direct(hrt_context *ctx, const hrt_launch *p) {
    if (!ctx || !p) return HRT_EINVAL;
    int r = check_built(ctx);
    if (r) return r;
    if (!p->band_launch_flag) return fail(ctx, HRT_EINVAL, "null band_launch_flag");
    if (p->launch_offset + (uint64_t)p->launch_count > (uint64_t)ctx->n)
        return fail(ctx, HRT_EINVAL, "launch range exceeds the primitive count");
    int Bg = (int)p->nbands_global, Bl = (int)p->nbands_launch;
    int Bc = count_flags(Bg, p->band_launch_flag);
    if (Bl != ctx->Bl) return fail(ctx, HRT_EINVAL, "nbands_launch differs from the last hrt_zero_radiation_buffers()");
    if (Bg > ctx->mB) return fail(ctx, HRT_EINVAL, "nbands_global exceeds the band count of the materials");
    if ((r = upload_flags(ctx, Bg, p->band_launch_flag))) return r;
    CU(cudaMemsetAsync(ctx->counter.p, 0, sizeof(unsigned long long), ctx->stream));
    if ((r = direct_pass(ctx, p->launch_offset, p->launch_count, p->rays_per_primitive, p->random_seed, p->pass_id, Bg, Bc, Bl)))
        return r;
    return sync_and_status(ctx);
}

int hrt_launch_diffuse(hrt_context *ctx, const hrt_launch *p) {
    if (!ctx || !p) return HRT_EINVAL;
    int r = check_built(ctx);
    if (r) return r;
    if (!p->band_launch_flag) return fail(ctx, HRT_EINVAL, "null band_launch_flag");
    if (p->launch_offset + (uint64_t)p->launch_count > (uint64_t)ctx->n)
        return fail(ctx, HRT_EINVAL, "launch range exceeds the primitive count");
    int Bg = (int)p->nbands_global, Bl = (int)p->nbands_launch;
    if (Bl != ctx->Bl) return fail(ctx, HRT_EINVAL, "nbands_launch differs from the last hrt_zero_radiation_buffers()");
    if (Bg > ctx->mB) return fail(ctx, HRT_EINVAL, "nbands_global exceeds the band count of the materials");
    size_t m = (size_t)ctx->n * Bl;
    // OptiX8Backend.cpp:887-898: radiation_out is uploaded before the launch when given.
    if (p->radiation_out_top) CU(cudaMemcpyAsync(ctx->otop.p, p->radiation_out_top, m * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    if (p->radiation_out_bottom) CU(cudaMemcpyAsync(ctx->obot.p, p->radiation_out_bottom, m * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    if (p->rays_per_primitive == 0 || p->launch_count == 0) return sync_and_status(ctx);
    int Bc = count_flags(Bg, p->band_launch_flag);
    if ((r = upload_flags(ctx, Bg, p->band_launch_flag))) return r;
    SkyParams sky;
    if ((r = upload_sky(ctx, Bl, p->diffuse_flux, p->diffuse_extinction, p->diffuse_dist_norm, p->diffuse_peak_dir,
                        p->sky_radiance_params, &sky)))
        return r;
    CU(cudaMemsetAsync(ctx->counter.p, 0, sizeof(unsigned long long), ctx->stream));
    int faces = (p->launch_face == 1) ? 1 : 2;
    if ((r = diffuse_pass(ctx, p->launch_offset, p->launch_count, p->rays_per_primitive, p->random_seed, p->pass_id,
                          faces, Bg, Bc, Bl, sky)))
        return r;
    return sync_and_status(ctx);
}

int hrt_query_memory(hrt_context *ctx, size_t *free_bytes, size_t *total_bytes) {
    if (!ctx) return HRT_EINVAL;
    CU(cudaSetDevice(ctx->device));
    size_t f = 0, t = 0;
    CU(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return HRT_OK;
}

// ------------------------------------------------------------ runBand ----
int hrt_run_band(hrt_context *ctx, const hrt_band_solve *s, float *flux_out) {
    if (!ctx || !s) return HRT_EINVAL;
    int r = check_built(ctx);
    if (r) return r;
    CU(cudaSetDevice(ctx->device));
    const int n = ctx->n, Bg = s->nbands_global;
    if (!s->band_launch || Bg <= 0) return fail(ctx, HRT_EINVAL, "no bands");
    const int Bl = count_flags(Bg, s->band_launch);
    if (Bl == 0) return fail(ctx, HRT_EINVAL, "no band is launched");
    if (Bl > 16) return fail(ctx, HRT_EUNSUPPORTED, "at most 16 bands per runBand");
    if (!s->direct_rays || !s->diffuse_rays || !s->scattering_depth || !s->emission || !s->diffuse_flux)
        return fail(ctx, HRT_EINVAL, "null per-band array");
    ctx->last_kernels = 0;
    int iters = 0;
    if (!(s->scatter_tolerance >= 0.0)) return fail(ctx, HRT_EINVAL, "scatter_tolerance must be >= 0");
    // materials / sources: NULL keeps what is resident on the device
    if (s->rho || s->tau) {
        if (!s->rho || !s->tau) return fail(ctx, HRT_EINVAL, "rho and tau must be given together");
        if ((r = hrt_update_materials(ctx, std::max(s->nsources, 1), n, Bg, s->rho, s->tau))) return r;
    }
    if (s->sources) {
        if ((r = hrt_update_sources(ctx, s->nsources, s->sources))) return r;
    }
    if (s->source_flux && s->nsources > 0) {
        if ((r = hrt_upload_source_fluxes(ctx, s->source_flux, (size_t)s->nsources * Bl))) return r;
    }
    if (ctx->mN != n || ctx->mB < Bg || ctx->mS < 1) return fail(ctx, HRT_EINVAL, "materials do not match the scene");
    const int S = ctx->S;
    bool rundirect = false;
    if (ctx->h_src_flux.size() < (size_t)S * Bl)
        return fail(ctx, HRT_EINVAL, "source fluxes not set for every source and launched band");
    for (size_t i = 0; i < (size_t)S * Bl; ++i) rundirect = rundirect || ctx->h_src_flux[i] > 0.f;
    bool scattering = false, diffuse = false, emission = false;
    int dirN = 0, difN = 0, depth = 0;
    for (int b = 0; b < Bl; ++b) {
        scattering = scattering || s->scattering_depth[b] > 0;
        diffuse = diffuse || s->diffuse_flux[b] > 0.f;
        emission = emission || s->emission[b];
        dirN = std::max(dirN, s->direct_rays[b]);
        difN = std::max(difN, s->diffuse_rays[b]);
        depth = std::max(depth, s->scattering_depth[b]);
    }
    if ((r = ensure_buffers(ctx, Bl))) return r;
    ctx->Bl = Bl;
    const size_t m = (size_t)n * Bl;
    cudaStream_t st = ctx->stream;
    CU(cudaMemsetAsync(ctx->rin.p, 0, m * sizeof(double), st));
    CU(cudaMemsetAsync(ctx->stop.p, 0, m * sizeof(double), st));
    CU(cudaMemsetAsync(ctx->sbot.p, 0, m * sizeof(double), st));
    CU(cudaMemsetAsync(ctx->ftop.p, 0, m * sizeof(double), st));
    CU(cudaMemsetAsync(ctx->fbot.p, 0, m * sizeof(double), st));
    CU(cudaMemsetAsync(ctx->otop.p, 0, m * sizeof(float), st));
    CU(cudaMemsetAsync(ctx->obot.p, 0, m * sizeof(float), st));
    CU(cudaMemsetAsync(ctx->counter.p, 0, sizeof(unsigned long long), st));
    std::vector<uint8_t> flags(s->band_launch, s->band_launch + Bg);
    if ((r = upload_flags(ctx, Bg, flags.data()))) return r;
    // Camera view of the primitives: the scatter of every pass plus emission, accumulated
    // (RadiationModel.cpp:3992-4012, 4105-4131, 4211-4220, 4336-4345).
    const bool cams = s->ncameras > 0 && s->cameras;
    ctx->cam_id_cur = 0xFFFFFFFFu;
    if (cams) {
        CU(ctx->ctop.ensure(st, m * sizeof(double)));
        CU(ctx->cbot.ensure(st, m * sizeof(double)));
        CU(cudaMemsetAsync(ctx->ctop.p, 0, m * sizeof(double), st));
        CU(cudaMemsetAsync(ctx->cbot.p, 0, m * sizeof(double), st));
    }
    auto cam_add_scatter = [&]() -> int {
        if (!cams) return HRT_OK;
        CU(launch_add(ctx->ctop.as<double>(), ctx->stop.as<double>(), m, st));
        CU(launch_add(ctx->cbot.as<double>(), ctx->sbot.as<double>(), m, st));
        ctx->last_kernels += 2;
        return HRT_OK;
    };
    if (emission) {
        // per-band flags and depths (small, every call); emissivity and temperature when given,
        // else the arrays resident from an earlier call are used
        if (Bl > 15) return fail(ctx, HRT_EUNSUPPORTED, "emission supports at most 15 launched bands");
        CU(ctx->emis.ensure(ctx->stream, 128));
        CU(cudaMemcpyAsync(ctx->emis.p, s->emission, (size_t)Bl, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(ctx->emis.as<char>() + 64, s->scattering_depth, (size_t)Bl * 4, cudaMemcpyHostToDevice, st));
        if (s->emissivity) {
            CU(ctx->emis_eps.ensure(ctx->stream, m * sizeof(float)));
            CU(cudaMemcpyAsync(ctx->emis_eps.p, s->emissivity, m * sizeof(float), cudaMemcpyHostToDevice, st));
            ctx->emis_eps_count = m;
        }
        if (s->temperature) {
            CU(ctx->emis_T.ensure(ctx->stream, (size_t)n * sizeof(float)));
            CU(cudaMemcpyAsync(ctx->emis_T.p, s->temperature, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st));
            ctx->emis_T_count = (size_t)n;
        }
        if (ctx->emis_eps_count != m || ctx->emis_T_count != (size_t)n)
            return fail(ctx, HRT_EINVAL, "emission needs emissivity [n*Bl] and temperature [n]");
    }
    // ---- direct
    if (S > 0 && rundirect && dirN > 0) {
        if ((r = direct_pass(ctx, 0, (uint32_t)n, (uint32_t)dirN, s->seed, 0u, Bg, Bl, Bl))) return r;
    }
    // ---- scattered direct energy becomes the outgoing flux (one-sided prims fold top+bottom)
    if (scattering && rundirect) {
        if ((r = cam_add_scatter())) return r;
        CU(launch_fold_onesided(n, Bl, ctx->twosided.as<int8_t>(), ctx->stop.as<double>(), ctx->sbot.as<double>(),
                                ctx->ftop.as<double>(), ctx->fbot.as<double>(), st));
        CU(cudaMemsetAsync(ctx->stop.p, 0, m * sizeof(double), st));
        CU(cudaMemsetAsync(ctx->sbot.p, 0, m * sizeof(double), st));
        ctx->last_kernels += 1;
    }
    uint32_t rpp_d = 0;
    {
        double c = std::ceil(std::sqrt((double)difN));
        rpp_d = (uint32_t)(c * c);
    }
    SkyParams sky;
    if ((r = upload_sky(ctx, Bl, s->diffuse_flux, s->diffuse_extinction, s->diffuse_dist_norm, s->diffuse_peak_dir,
                        s->sky_radiance_params, &sky)))
        return r;
    if (emission || diffuse) {
        if (emission) {
            CU(launch_emission(n, Bl, ctx->emis.as<uint8_t>(), (const int32_t *)(ctx->emis.as<char>() + 64),
                               ctx->emis_eps.as<float>(), ctx->emis_T.as<float>(), ctx->twosided.as<int8_t>(),
                               ctx->ftop.as<double>(), ctx->fbot.as<double>(), st));
            ctx->last_kernels += 1;
            if (cams) {
                CU(launch_emission(n, Bl, ctx->emis.as<uint8_t>(), (const int32_t *)(ctx->emis.as<char>() + 64),
                                   ctx->emis_eps.as<float>(), ctx->emis_T.as<float>(), ctx->twosided.as<int8_t>(),
                                   ctx->ctop.as<double>(), ctx->cbot.as<double>(), st));
                ctx->last_kernels += 1;
            }
        }
        CU(launch_to_float(ctx->ftop.as<double>(), ctx->otop.as<float>(), m, st));
        CU(launch_to_float(ctx->fbot.as<double>(), ctx->obot.as<float>(), m, st));
        ctx->last_kernels += 2;
        if ((r = diffuse_pass(ctx, 0, (uint32_t)n, rpp_d, s->seed, 1u, 3, Bg, Bl, Bl, sky))) return r;
        if ((r = cam_add_scatter())) return r;
    } else if (scattering && rundirect) {
        CU(launch_to_float(ctx->ftop.as<double>(), ctx->otop.as<float>(), m, st));
        CU(launch_to_float(ctx->fbot.as<double>(), ctx->obot.as<float>(), m, st));
        ctx->last_kernels += 2;
    }
    if (scattering && (emission || diffuse) && !rundirect) {
        CU(launch_to_float(ctx->stop.as<double>(), ctx->otop.as<float>(), m, st));
        CU(launch_to_float(ctx->sbot.as<double>(), ctx->obot.as<float>(), m, st));
        CU(cudaMemsetAsync(ctx->stop.p, 0, m * sizeof(double), st));
        CU(cudaMemsetAsync(ctx->sbot.p, 0, m * sizeof(double), st));
        ctx->last_kernels += 2;
    }
    if (scattering && (emission || diffuse || rundirect)) {
        std::vector<float> zero((size_t)Bl, 0.f);
        SkyParams sky0;
        {
            // zero diffuse flux for the scattering iterations (RadiationModel.cpp:4237-4240)
            CU(cudaMemsetAsync((void *)sky.flux, 0, (size_t)Bl * sizeof(float), st));
            sky0 = sky;
        }
        std::vector<uint8_t> sflags = flags, conv(Bg, 0);
        const bool residual = s->scatter_tolerance > 0.0;
        if (residual) CU(ctx->resid.ensure(ctx->stream, (64 + (size_t)kResidualBlocks * Bl * 2) * sizeof(double)));
        for (int it = 0; it < depth; ++it) {
            int b = -1;
            for (int bg = 0; bg < Bg; ++bg) {
                if (!sflags[bg]) continue;
                ++b;
                if (it + 1 > s->scattering_depth[b] || conv[bg]) sflags[bg] = 0;
            }
            if ((r = upload_flags(ctx, Bg, sflags.data()))) return r;
            if (it > 0 || (emission && rundirect)) {
                CU(launch_to_float(ctx->stop.as<double>(), ctx->otop.as<float>(), m, st));
                CU(launch_to_float(ctx->sbot.as<double>(), ctx->obot.as<float>(), m, st));
                ctx->last_kernels += 2;
            }
            CU(cudaMemsetAsync(ctx->stop.p, 0, m * sizeof(double), st));
            CU(cudaMemsetAsync(ctx->sbot.p, 0, m * sizeof(double), st));
            int Bc = count_flags(Bg, sflags.data());
            if ((r = diffuse_pass(ctx, 0, (uint32_t)n, rpp_d, s->seed, 2u + (uint32_t)it, 3, Bg, Bc, Bl, sky0))) return r;
            if ((r = cam_add_scatter())) return r;
            iters = it + 1;
            if (residual) {
                // FP64 convergence check: a band stops once the power its last iteration
                // scattered (not yet propagated) is at most scatter_tolerance of its total.
                double h[32];
                CU(launch_residual(n, Bl, ctx->area.as<double>(), ctx->rin.as<double>(), ctx->stop.as<double>(),
                                   ctx->sbot.as<double>(), ctx->resid.as<double>(), st));
                CU(cudaMemcpyAsync(h, ctx->resid.p, 2 * (size_t)Bl * sizeof(double), cudaMemcpyDeviceToHost, st));
                CU(cudaStreamSynchronize(st));
                ctx->last_kernels += 2;
                bool all = true;
                int c = -1;
                for (int bg = 0; bg < Bg; ++bg) {
                    if (!flags[bg]) continue;
                    ++c;
                    if (!sflags[bg]) continue;
                    if (h[2 * c] <= s->scatter_tolerance * h[2 * c + 1]) conv[bg] = 1;
                    else all = false;
                }
                if (all) break;
            }
        }
    }
    CU(launch_final_flux(m, ctx->rin.as<double>(), ctx->stop.as<double>(), ctx->sbot.as<double>(), ctx->fin.as<float>(), st));
    ctx->last_kernels += 1;
    if (flux_out) CU(cudaMemcpyAsync(flux_out, ctx->fin.p, m * sizeof(float), cudaMemcpyDeviceToHost, st));
    // ---- cameras (RadiationModel.cpp:4358-4616), rendered from the accumulated camera view
    if (cams) {
        const bool render = scattering && (emission || diffuse || rundirect);
        if (render) {
            if ((r = hrt_update_sky_model(ctx, s->camera_sky ? Bl : 0, s->camera_sky))) return r;
            CU(launch_to_float(ctx->ctop.as<double>(), ctx->otop.as<float>(), m, st));
            CU(launch_to_float(ctx->cbot.as<double>(), ctx->obot.as<float>(), m, st));
            ctx->last_kernels += 2;
        }
        for (int ci = 0; ci < s->ncameras; ++ci) {
            hrt_camera c = s->cameras[ci];
            c.tile_offset[0] = c.tile_offset[1] = 0;
            c.tile_resolution[0] = c.tile_resolution[1] = 0;
            CameraParams P;
            if ((r = camera_params(ctx, &c, Bl, &P))) return r;
            const size_t npx = (size_t)P.W * P.H;
            if ((r = ensure_camera_image(ctx, P.W, P.H, Bl))) return r;
            if ((r = ensure_camera_labels(ctx, P.W, P.H))) return r;
            ctx->cam_id_cur = c.camera_id;
            P.pix = ctx->cam_pix.as<double>();
            P.labels = ctx->cam_lab.as<uint32_t>();
            P.depths = ctx->cam_dep.as<float>();
            if (render) {
                CU(launch_camera(P, max_blocks(ctx), st));
                CU(launch_pixel_labels(P, st));
                ctx->last_kernels += 2;
            }
            if (c.pixels) {
                CU(ctx->io_a.ensure(st, npx * Bl * sizeof(float)));
                CU(launch_to_float(ctx->cam_pix.as<double>(), ctx->io_a.as<float>(), npx * Bl, st));
                CU(cudaMemcpyAsync(c.pixels, ctx->io_a.p, npx * Bl * sizeof(float), cudaMemcpyDeviceToHost, st));
                CU(cudaStreamSynchronize(st));
            }
            if (c.labels) CU(cudaMemcpyAsync(c.labels, ctx->cam_lab.p, npx * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
            if (c.depths) CU(cudaMemcpyAsync(c.depths, ctx->cam_dep.p, npx * sizeof(float), cudaMemcpyDeviceToHost, st));
        }
    }
    unsigned long long rays = 0;
    CU(cudaMemcpyAsync(&rays, ctx->counter.p, sizeof(rays), cudaMemcpyDeviceToHost, st));
    r = sync_and_status(ctx);
    ctx->last_rays = rays;
    ctx->last_iters = (uint64_t)iters;
    return r;
}

// ------------------------------------------------------------ batched sweep --
}  // extern "C"

namespace {

// A sweep of one scene, prepared for capture: inputs uploaded, buffers sized, the pass
// sequence's flags and the recording kernel's variant chosen.
struct SweepPlan {
    hrt_context *ctx = nullptr;
    int n = 0, nsun = 0, Bl = 0, C = 0;
    size_t m = 0;
    bool scattering = false, any_direct = false, any_diffuse = false, any_copy0 = false, any_active = false;
    int dimx = 0, dimy = 0, ddx = 0, ddy = 0, Rd = 0, depth = 0;
    uint32_t seed = 0, rec_per = 0;
    int rec_variant = DV_W4;
    float *d_sun = nullptr, *d_flux = nullptr, *d_sky = nullptr, *d_zero = nullptr;
    uint8_t *m_all = nullptr, *m_fold = nullptr, *m_diff = nullptr, *m_copy0 = nullptr, *m_active = nullptr;
    float *d_rho = nullptr, *d_tau = nullptr;
    double *rin = nullptr, *stp = nullptr, *sbt = nullptr, *Gt = nullptr, *Gb = nullptr;
    float *otop = nullptr, *obot = nullptr, *fin = nullptr;
    uint32_t *hits = nullptr;
    bool traces_diffuse() const { return Rd > 0 && any_diffuse; }
    bool traces_scatter(int it) const { return Rd > 0 && scattering && any_active && it < depth; }
};

// Validates the sweep, uploads its inputs on the context's stream and sizes its buffers.
// tune: time the recording kernel's variants (not allowed while another graph is captured).
int sweep_prepare(hrt_context *ctx, const hrt_sweep *s, bool tune, SweepPlan *pl) {
    if (!ctx || !s) return HRT_EINVAL;
    int r = check_built(ctx);
    if (r) return r;
    CU(cudaSetDevice(ctx->device));
    if (!ctx->h_voxels.empty()) return fail(ctx, HRT_EUNSUPPORTED, "the batched sweep does not trace voxels");
    if (ctx->gS > 0) return fail(ctx, HRT_EUNSUPPORTED, "the batched sweep does not trace translucent covers");
    const int n = ctx->n, nsun = s->nsun, Bl = s->nbands;
    if (nsun < 1 || Bl < 1 || !s->sun_dir || !s->direct_flux || !s->diffuse_flux || !s->rho || !s->tau)
        return fail(ctx, HRT_EINVAL, "sweep needs suns, bands, fluxes and materials");
    const int C = nsun * Bl;
    if (C > 256) return fail(ctx, HRT_EUNSUPPORTED, "a sweep holds at most 256 channels");
    if (s->direct_rays < 0 || s->diffuse_rays < 0 || s->scattering_depth < 0) return fail(ctx, HRT_EINVAL, "negative count");
    SweepPlan P;
    P.ctx = ctx;
    P.n = n;
    P.nsun = nsun;
    P.Bl = Bl;
    P.C = C;
    P.m = (size_t)n * C;
    P.depth = s->scattering_depth;
    P.seed = s->seed;
    cudaStream_t st = ctx->stream;
    // per-channel pass-sequence flags of the plain runBand each channel stands for
    P.scattering = s->scattering_depth > 0;
    std::vector<uint8_t> all(C, 1), rundirect(C), diffuse(C), fold(C), copy0(C), active(C);
    for (int c = 0; c < C; ++c) {
        rundirect[c] = s->direct_flux[c] > 0.f;
        diffuse[c] = s->diffuse_flux[c] > 0.f;
        fold[c] = P.scattering && rundirect[c];
        copy0[c] = P.scattering && diffuse[c] && !rundirect[c];
        active[c] = diffuse[c] || rundirect[c];
        P.any_direct = P.any_direct || rundirect[c];
        P.any_diffuse = P.any_diffuse || diffuse[c];
        P.any_copy0 = P.any_copy0 || copy0[c];
        P.any_active = P.any_active || active[c];
    }
    strata((uint32_t)s->direct_rays, &P.dimx, &P.dimy);
    uint32_t rpp_d;
    {
        double c = std::ceil(std::sqrt((double)s->diffuse_rays));
        rpp_d = (uint32_t)(c * c);
    }
    strata(rpp_d, &P.ddx, &P.ddy);
    P.Rd = P.ddx * P.ddy;
    // device inputs: [sun 3*nsun][flux C][sky C][zero C] floats, masks 6*C bytes, materials
    CU(ctx->sw_in.ensure(ctx->stream, (3 * (size_t)nsun + 3 * (size_t)C) * sizeof(float) + 6 * (size_t)C + 256));
    P.d_sun = ctx->sw_in.as<float>();
    P.d_flux = P.d_sun + 3 * nsun;
    P.d_sky = P.d_flux + C;
    P.d_zero = P.d_sky + C;
    uint8_t *d_masks = (uint8_t *)(P.d_zero + C);
    {
        std::vector<float> h(3 * (size_t)nsun + 3 * (size_t)C, 0.f);
        std::copy(s->sun_dir, s->sun_dir + 3 * nsun, h.begin());
        std::copy(s->direct_flux, s->direct_flux + C, h.begin() + 3 * nsun);
        std::copy(s->diffuse_flux, s->diffuse_flux + C, h.begin() + 3 * nsun + C);
        std::vector<uint8_t> mk8;
        for (auto *v : {&all, &fold, &diffuse, &copy0, &active, &rundirect}) mk8.insert(mk8.end(), v->begin(), v->end());
        CU(cudaMemcpyAsync(P.d_sun, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(d_masks, mk8.data(), mk8.size(), cudaMemcpyHostToDevice, st));
    }
    P.m_all = d_masks;
    P.m_fold = d_masks + C;
    P.m_diff = d_masks + 2 * C;
    P.m_copy0 = d_masks + 3 * C;
    P.m_active = d_masks + 4 * C;
    CU(ctx->sw_mat.ensure(ctx->stream, 2 * (size_t)n * Bl * sizeof(float)));
    P.d_rho = ctx->sw_mat.as<float>();
    P.d_tau = P.d_rho + (size_t)n * Bl;
    CU(cudaMemcpyAsync(P.d_rho, s->rho, (size_t)n * Bl * sizeof(float), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P.d_tau, s->tau, (size_t)n * Bl * sizeof(float), cudaMemcpyHostToDevice, st));
    // buffers
    const size_t m = P.m;
    CU(ctx->sw_acc.ensure(ctx->stream, 5 * m * sizeof(double)));
    P.rin = ctx->sw_acc.as<double>();
    P.stp = P.rin + m;
    P.sbt = P.stp + m;
    P.Gt = P.sbt + m;
    P.Gb = P.Gt + m;
    CU(ctx->sw_out.ensure(ctx->stream, 3 * m * sizeof(float)));
    P.otop = ctx->sw_out.as<float>();
    P.obot = P.otop + m;
    P.fin = P.obot + m;
    const size_t nhits = 2 * (size_t)n * (size_t)std::max(P.Rd, 1);
    // recording launches over primitive chunks of at most rec_per primitives (32-bit ray ids)
    P.rec_per = chunk_prims(ctx, 2ull * (uint64_t)std::max(P.Rd, 1));
    if (P.rec_per == 0) return HRT_EUNSUPPORTED;
    if ((uint64_t)n * (uint64_t)nsun >= 0xFFFFFFFFull)  // (primitive, sun) sum keys are 32-bit
        return fail(ctx, HRT_EUNSUPPORTED, "primitives x suns of a sweep must stay below 2^32");
    CU(ctx->sw_hits.ensure(ctx->stream, nhits * sizeof(uint32_t)));
    P.hits = ctx->sw_hits.as<uint32_t>();
    CU(ctx->Gd.ensure(ctx->stream, std::max<size_t>((size_t)n * nsun * 2, 1) * sizeof(double)));
    CU(ctx->fetch.ensure(ctx->stream, sizeof(unsigned long long)));
    // choose the recording kernel's variant before capture (timing cannot run inside a capture)
    P.rec_variant = ctx->n4 > 0 ? DV_W4 : DV_PS3;
    if (tune && P.Rd > 0 && (P.any_diffuse || P.any_active)) {
        DiffuseParams T0{};
        T0.sc = scene_of(ctx);
        T0.dimx = P.ddx;
        T0.dimy = P.ddy;
        T0.seed = s->seed;
        T0.pass = 1;
        T0.count = (uint32_t)n;
        T0.faces = 3;
        T0.Bc = 1;
        T0.Bl = 1;
        T0.fetch = ctx->fetch.as<unsigned long long>();
        T0.lane_budget = ctx->lane_budget;
        T0.hits = P.hits;
        if ((r = tuned_variant(ctx, T0, true, &P.rec_variant))) return r;
    }
    *pl = P;
    return HRT_OK;
}

// Shape and buffers of a prepared sweep: a captured graph is valid while these stay the same.
std::string sweep_key(const SweepPlan &P, const hrt_sweep *s) {
    hrt_context *ctx = P.ctx;
    char key[384];
    std::snprintf(key, sizeof key, "%d/%d/%d/%d/%d/%d/%u/%d%d%d%d/%p/%p/%p/%p/%p/%p/%p/v%d/c%u", P.n, P.nsun, P.Bl,
                  s->direct_rays, s->diffuse_rays, s->scattering_depth, s->seed, (int)P.any_direct,
                  (int)P.any_diffuse, (int)P.any_copy0, (int)P.any_active, ctx->sw_acc.p, ctx->sw_hits.p,
                  ctx->sw_in.p, ctx->sw_mat.p, ctx->sw_out.p, ctx->Gd.p, (void *)ctx->stream, P.rec_variant,
                  P.rec_per);
    return key;
}

// Capture-safe stages of a sweep, queued on st.
struct SweepStages {
    const SweepPlan &P;
    cudaStream_t st;
    int &nk;  // kernels queued

    ChannelEpilogue epilogue() const {
        ChannelEpilogue E{};
        E.n = P.n;
        E.C = P.C;
        E.Bl = P.Bl;
        E.rho = P.d_rho;
        E.tau = P.d_tau;
        E.rin = P.rin;
        E.stop = P.stp;
        E.sbot = P.sbt;
        E.Gt = P.Gt;
        E.Gb = P.Gb;
        E.strength = 1.0 / (double)std::max(P.Rd, 1);
        return E;
    }
    DiffuseParams record_params(uint32_t pass) const {
        DiffuseParams D{};
        TraceScene sc = scene_of(P.ctx);
        sc.visits = nullptr;
        D.sc = sc;
        D.dimx = P.ddx;
        D.dimy = P.ddy;
        D.seed = P.seed;
        D.pass = pass;
        D.offset = 0;
        D.count = (uint32_t)P.n;
        D.faces = 3;
        D.fetch = P.ctx->fetch.as<unsigned long long>();
        D.lane_budget = P.ctx->lane_budget;
        return D;
    }
    // accumulators and the ray counter to zero, the direct pass per sun, the one-sided fold
    cudaError_t begin() {
        cudaError_t e;
        hrt_context *ctx = P.ctx;
        if ((e = cudaMemsetAsync(P.rin, 0, 3 * P.m * sizeof(double), st)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(ctx->counter.p, 0, sizeof(unsigned long long), st)) != cudaSuccess) return e;
        if (P.any_direct && P.dimx * P.dimy > 0) {
            if ((e = cudaMemsetAsync(ctx->Gd.p, 0, (size_t)P.n * P.nsun * 2 * sizeof(double), st)) != cudaSuccess)
                return e;
            TraceScene sc = scene_of(ctx);
            sc.visits = nullptr;
            SweepDirectParams D{sc, P.d_sun, P.nsun, P.dimx, P.dimy, P.seed, ctx->Gd.as<double>()};
            if ((e = launch_direct_sweep(D, max_blocks(ctx), st)) != cudaSuccess) return e;
            ChannelEpilogue E = epilogue();
            E.flux = P.d_flux;
            E.mask = P.m_all;
            E.Gd = ctx->Gd.as<double>();
            if ((e = launch_epilogue_direct_channels(E, st)) != cudaSuccess) return e;
            nk += 2;
        }
        if ((e = launch_fold_channels(P.n, P.C, P.m_fold, scene_of(ctx).twosided, P.stp, P.sbt, P.otop, P.obot, st)) !=
            cudaSuccess)
            return e;
        ++nk;
        return cudaSuccess;
    }
    // this scene's recording launches of one pass (primitive chunks of the plan)
    cudaError_t record(uint32_t pass) {
        DiffuseParams Q = record_params(pass);
        for (uint32_t done = 0; done < (uint32_t)P.n; done += Q.count) {
            Q.offset = done;
            Q.count = std::min(P.rec_per, (uint32_t)P.n - done);
            cudaError_t e = launch_diffuse_record(Q, P.hits, P.rec_variant, st);
            if (e != cudaSuccess) return e;
            ++nk;
        }
        return cudaSuccess;
    }
    // channel gather of the recorded hits and the pass's epilogue
    cudaError_t gather(const float *sky, const uint8_t *mask) {
        cudaError_t e;
        GatherParams Gp{P.n, P.C, P.Rd, 3, scene_of(P.ctx).twosided, P.hits, P.otop, P.obot, sky, P.Gt, P.Gb};
        if ((e = launch_gather(Gp, st)) != cudaSuccess) return e;
        ChannelEpilogue E = epilogue();
        E.mask = mask;
        if ((e = launch_epilogue_diffuse_channels(E, st)) != cudaSuccess) return e;
        nk += 2;
        return cudaSuccess;
    }
    cudaError_t after_primary() {
        if (!P.any_copy0) return cudaSuccess;
        ++nk;
        return launch_copy_channels(P.n, P.C, P.m_copy0, P.stp, P.sbt, P.otop, P.obot, 1, st);
    }
    // before scattering iteration it: scatter -> radiation_out (it > 0), scatter sums to zero
    cudaError_t before_scatter(int it) {
        cudaError_t e;
        if (it > 0) {
            if ((e = launch_copy_channels(P.n, P.C, P.m_all, P.stp, P.sbt, P.otop, P.obot, 0, st)) != cudaSuccess)
                return e;
            ++nk;
        }
        return cudaMemsetAsync(P.stp, 0, 2 * P.m * sizeof(double), st);
    }
    cudaError_t finish() {
        ++nk;
        return launch_final_flux(P.m, P.rin, P.stp, P.sbt, P.fin, st);
    }
};

// Capture `enqueue` on st into *exec (replacing the old graph).
template <class F>
int capture_graph(hrt_context *ctx, cudaStream_t st, cudaGraphExec_t *exec, F &&enqueue) {
    if (*exec) {
        cudaGraphExecDestroy(*exec);
        *exec = nullptr;
    }
    CU(cudaStreamSynchronize(st));
    CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t ee = enqueue();
    cudaGraph_t g = nullptr;
    cudaError_t ec = cudaStreamEndCapture(st, &g);
    if (ee != cudaSuccess || ec != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(ctx, HRT_ECUDA, std::string("sweep capture failed: ") + cudaGetErrorString(ee != cudaSuccess ? ee : ec));
    }
    cudaError_t ei = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return fail(ctx, HRT_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
    return HRT_OK;
}

}  // namespace

extern "C" {

int hrt_run_sweep(hrt_context *ctx, const hrt_sweep *s, float *flux_out) {
    SweepPlan P;
    int r = sweep_prepare(ctx, s, true, &P);
    if (r) return r;
    cudaStream_t st = ctx->stream;
    // capture the pass sequence once per shape
    const std::string key = sweep_key(P, s);
    if (!ctx->sw_exec || ctx->sw_key != key) {
        int nk = 0;
        SweepStages S{P, st, nk};
        r = capture_graph(ctx, st, &ctx->sw_exec, [&]() -> cudaError_t {
            cudaError_t e;
            if ((e = S.begin()) != cudaSuccess) return e;
            if (P.traces_diffuse()) {
                if ((e = S.record(1u)) != cudaSuccess || (e = S.gather(P.d_sky, P.m_diff)) != cudaSuccess) return e;
            }
            if ((e = S.after_primary()) != cudaSuccess) return e;
            for (int it = 0; P.traces_scatter(it); ++it) {
                if ((e = S.before_scatter(it)) != cudaSuccess || (e = S.record(2u + (uint32_t)it)) != cudaSuccess ||
                    (e = S.gather(P.d_zero, P.m_active)) != cudaSuccess)
                    return e;
            }
            return S.finish();
        });
        if (r) return r;
        ctx->sw_key = key;
        ctx->sw_kernels = nk;
    }
    CU(cudaGraphLaunch(ctx->sw_exec, st));
    ctx->last_kernels = ctx->sw_kernels;
    if (flux_out) CU(cudaMemcpyAsync(flux_out, P.fin, P.m * sizeof(float), cudaMemcpyDeviceToHost, st));
    unsigned long long rays = 0;
    CU(cudaMemcpyAsync(&rays, ctx->counter.p, sizeof(rays), cudaMemcpyDeviceToHost, st));
    r = sync_and_status(ctx);
    ctx->last_rays = rays;
    ctx->last_iters = (uint64_t)s->scattering_depth;
    return r;
}

int hrt_run_sweep_multi(hrt_context *const *ctxs, const hrt_sweep *sweeps, int32_t nscenes, float *const *flux_out) {
    if (!ctxs || !sweeps || nscenes < 1 || !ctxs[0]) return HRT_EINVAL;
    hrt_context *ctx = ctxs[0];  // owns the graph and the slot tables; its stream runs the graph
    for (int k = 0; k < nscenes; ++k) {
        if (!ctxs[k]) return fail(ctx, HRT_EINVAL, "null context in a multi-scene sweep");
        if (ctxs[k]->device != ctx->device) return fail(ctx, HRT_EINVAL, "the scenes of a multi-scene sweep share one device");
        for (int j = 0; j < k; ++j)
            if (ctxs[j] == ctxs[k]) return fail(ctx, HRT_EINVAL, "a context appears twice in a multi-scene sweep");
    }
    std::vector<SweepPlan> plans(nscenes);
    std::string key = "multi";
    int r;
    for (int k = 0; k < nscenes; ++k) {
        if ((r = sweep_prepare(ctxs[k], &sweeps[k], false, &plans[k]))) {
            if (k > 0) fail(ctx, r, std::string("scene ") + std::to_string(k) + ": " + ctxs[k]->err);
            return r;
        }
        if (ctxs[k]->n4 <= 0) return fail(ctx, HRT_EUNSUPPORTED, "multi-scene sweeps trace 4-wide trees");
        key += "|" + sweep_key(plans[k], &sweeps[k]);
    }
    for (int k = 1; k < nscenes; ++k) CU(cudaStreamSynchronize(ctxs[k]->stream));  // their uploads
    cudaStream_t st = ctx->stream;
    // slot tables of the recording passes: pass 0 = primary diffuse, pass 1 + it = scattering it;
    // a pass lists the primitive chunks of every scene that traces it
    int maxdepth = 0;
    for (const auto &P : plans) maxdepth = std::max(maxdepth, P.depth);
    std::vector<SceneSlot> slots;
    std::vector<int> pass_first, pass_count;
    std::vector<unsigned long long> pass_total;
    for (int pass = 0; pass <= maxdepth; ++pass) {
        pass_first.push_back((int)slots.size());
        unsigned long long id = 0;
        for (const auto &P : plans) {
            if (!(pass == 0 ? P.traces_diffuse() : P.traces_scatter(pass - 1))) continue;
            for (uint32_t done = 0; done < (uint32_t)P.n; done += P.rec_per) {
                SceneSlot sl{};
                sl.sc = scene_of(P.ctx);
                sl.sc.visits = nullptr;
                sl.dimx = P.ddx;
                sl.dimy = P.ddy;
                sl.seed = P.seed;
                sl.pass = 1u + (uint32_t)pass;
                sl.offset = done;
                sl.count = std::min(P.rec_per, (uint32_t)P.n - done);
                sl.id_begin = id;
                sl.hits = P.hits;
                id += (unsigned long long)sl.count * (unsigned long long)P.Rd * 2ull;
                slots.push_back(sl);
            }
        }
        pass_count.push_back((int)slots.size() - pass_first.back());
        pass_total.push_back(id);
        if (pass_count.back() > kMaxSlots)
            return fail(ctx, HRT_EUNSUPPORTED, "a multi-scene pass holds at most 32 scene chunks");
    }
    CU(ctx->sw_slots.ensure(st, std::max<size_t>(slots.size(), 1) * sizeof(SceneSlot)));
    CU(cudaMemcpyAsync(ctx->sw_slots.p, slots.data(), slots.size() * sizeof(SceneSlot), cudaMemcpyHostToDevice, st));
    {
        char more[64];
        std::snprintf(more, sizeof more, "|slots %p %zu", ctx->sw_slots.p, slots.size());
        key += more;
    }
    if (!ctx->mw_exec || ctx->mw_key != key) {
        int nk = 0;
        std::vector<SweepStages> S;
        for (const auto &P : plans) S.push_back(SweepStages{P, st, nk});
        auto multi_record = [&](int pass) -> cudaError_t {
            if (pass_count[pass] == 0) return cudaSuccess;
            DiffuseParams D{};
            D.faces = 3;
            D.fetch = ctx->fetch.as<unsigned long long>();
            D.lane_budget = 0;
            D.slots = ctx->sw_slots.as<SceneSlot>() + pass_first[pass];
            D.nslots = pass_count[pass];
            D.multi_total = pass_total[pass];
            ++nk;
            return launch_w4s_multi_record(D, st);
        };
        r = capture_graph(ctx, st, &ctx->mw_exec, [&]() -> cudaError_t {
            cudaError_t e;
            for (auto &s : S)
                if ((e = s.begin()) != cudaSuccess) return e;
            if ((e = multi_record(0)) != cudaSuccess) return e;
            for (size_t k = 0; k < S.size(); ++k)
                if (plans[k].traces_diffuse() && (e = S[k].gather(plans[k].d_sky, plans[k].m_diff)) != cudaSuccess)
                    return e;
            for (auto &s : S)
                if ((e = s.after_primary()) != cudaSuccess) return e;
            for (int it = 0; it < maxdepth; ++it) {
                for (size_t k = 0; k < S.size(); ++k)
                    if (plans[k].traces_scatter(it) && (e = S[k].before_scatter(it)) != cudaSuccess) return e;
                if ((e = multi_record(1 + it)) != cudaSuccess) return e;
                for (size_t k = 0; k < S.size(); ++k)
                    if (plans[k].traces_scatter(it) && (e = S[k].gather(plans[k].d_zero, plans[k].m_active)) != cudaSuccess)
                        return e;
            }
            for (auto &s : S)
                if ((e = s.finish()) != cudaSuccess) return e;
            return cudaSuccess;
        });
        if (r) return r;
        ctx->mw_key = key;
        ctx->mw_kernels = nk;
    }
    CU(cudaGraphLaunch(ctx->mw_exec, st));
    std::vector<unsigned long long> rays(nscenes, 0);
    for (int k = 0; k < nscenes; ++k) {
        if (flux_out && flux_out[k])
            CU(cudaMemcpyAsync(flux_out[k], plans[k].fin, plans[k].m * sizeof(float), cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(&rays[k], ctxs[k]->counter.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    }
    CU(cudaStreamSynchronize(st));
    int status = HRT_OK;
    unsigned long long total = 0;
    for (int k = 0; k < nscenes; ++k) {
        ctxs[k]->last_rays = rays[k];
        ctxs[k]->last_iters = (uint64_t)sweeps[k].scattering_depth;
        ctxs[k]->last_kernels = ctx->mw_kernels;
        total += rays[k];
        uint32_t word = 0;  // each scene's device error word (the graph ran on ctx's stream)
        CU(cudaMemcpy(&word, ctxs[k]->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        if (word && status == HRT_OK) {
            int rk = sync_and_status(ctxs[k]);
            status = rk;
            if (k > 0) fail(ctx, rk, std::string("scene ") + std::to_string(k) + ": " + ctxs[k]->err);
        }
    }
    ctx->multi_rays = total;
    return status;
}

int hrt_set_launch_ray_limit(hrt_context *ctx, uint64_t max_rays) {
    if (!ctx || max_rays == 0) return HRT_EINVAL;
    ctx->ray_limit = std::min<uint64_t>(max_rays, kLaunchRayLimit);
    return HRT_OK;
}

int64_t hrt_plan_launch_chunks(uint32_t count, uint64_t rays_per_primitive, uint64_t max_rays,
                               uint32_t *prims_per_chunk) {
    if (max_rays == 0) max_rays = kLaunchRayLimit;
    const uint32_t per = launch_chunk_prims(rays_per_primitive, max_rays);
    if (prims_per_chunk) *prims_per_chunk = per;
    if (per == 0) return HRT_EUNSUPPORTED;
    if (count == 0) return 0;
    return (int64_t)(((uint64_t)count + per - 1) / per);
}

int hrt_set_visit_budget(hrt_context *ctx, uint32_t visits) {
    if (!ctx) return HRT_EINVAL;
    ctx->visit_budget = visits;
    return HRT_OK;
}

int hrt_set_ray_budget(hrt_context *ctx, uint32_t rays_per_thread) {
    if (!ctx || rays_per_thread > (1u << 20)) return HRT_EINVAL;
    ctx->lane_budget = rays_per_thread;
    ctx->tuned.clear();  // the budget changes the launches the tuner timed
    return HRT_OK;
}

int hrt_set_tuning(hrt_context *ctx, int mode) {
    if (!ctx || mode < 0 || (mode > 2 && !(mode >= 16 + DV_PS4 && mode <= 16 + DV_LAST))) return HRT_EINVAL;
    if (mode == 2) {
        ctx->tuned.clear();
        ctx->tune_log.clear();
        mode = 1;
    }
    ctx->tune = mode;
    return HRT_OK;
}

size_t hrt_tuning_report(const hrt_context *ctx, char *buf, size_t len) {
    if (!ctx) return 0;
    if (buf && len) {
        size_t k = std::min(len - 1, ctx->tune_log.size());
        std::memcpy(buf, ctx->tune_log.data(), k);
        buf[k] = 0;
    }
    return ctx->tune_log.size() + 1;
}

int hrt_last_stats(const hrt_context *ctx, uint64_t *stats, int count) {
    if (!ctx || !stats) return HRT_EINVAL;
    if (count > 0) stats[0] = ctx->last_rays;
    if (count > 1) stats[1] = ctx->last_kernels;
    if (count > 2) stats[2] = ctx->last_iters;
    if (count > 3) stats[3] = ctx->eb_unconverged;
    return HRT_OK;
}

int hrt_device_status(hrt_context *ctx, uint32_t *status, int reset) {
    if (!ctx || !status) return HRT_EINVAL;
    CU(cudaStreamSynchronize(ctx->stream));
    CU(cudaMemcpy(status, ctx->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (reset) CU(cudaMemset(ctx->status.p, 0, sizeof(uint32_t)));
    return HRT_OK;
}

// ------------------------------------------------------------ inspection --
int hrt_trace_rays(hrt_context *ctx, int64_t nrays, const float *origins, const float *dirs, float tmin, float tmax,
                   int anyhit, int32_t *hit, float *t, int32_t *face) {
    if (!ctx || nrays < 0 || (nrays && (!origins || !dirs || !hit || !t || !face))) return HRT_EINVAL;
    int r = check_built(ctx);
    if (r) return r;
    size_t nr = (size_t)nrays;
    CU(ctx->io_a.ensure(ctx->stream, std::max<size_t>(nr, 1) * 24));
    CU(ctx->io_b.ensure(ctx->stream, std::max<size_t>(nr, 1) * 12));
    float *dO = ctx->io_a.as<float>(), *dD = dO + 3 * nr;
    int32_t *dH = ctx->io_b.as<int32_t>();
    float *dT = (float *)(dH + nr);
    int32_t *dF = (int32_t *)(dT + nr);
    CU(cudaMemcpyAsync(dO, origins, nr * 12, cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaMemcpyAsync(dD, dirs, nr * 12, cudaMemcpyHostToDevice, ctx->stream));
    CU(launch_trace_rays(scene_of(ctx), nrays, dO, dD, tmin, tmax, anyhit, dH, dT, dF, ctx->stream));
    CU(cudaMemcpyAsync(hit, dH, nr * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaMemcpyAsync(t, dT, nr * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaMemcpyAsync(face, dF, nr * 4, cudaMemcpyDeviceToHost, ctx->stream));
    return sync_and_status(ctx);
}

int hrt_gen_rays(hrt_context *ctx, int kind, uint32_t seed, uint32_t pass, int32_t rpp, int32_t face,
                 const float *direction, float *origins, float *dirs) {
    if (!ctx || rpp < 0 || !origins || !dirs) return HRT_EINVAL;
    int r = check_built(ctx);
    if (r) return r;
    int dimx, dimy;
    strata((uint32_t)rpp, &dimx, &dimy);
    if (dimx < 1) {
        dimx = 1;
        dimy = rpp;
    }
    size_t nr = (size_t)ctx->n * dimx * dimy;
    CU(ctx->io_a.ensure(ctx->stream, std::max<size_t>(nr, 1) * 24));
    float *dO = ctx->io_a.as<float>(), *dD = dO + 3 * nr;
    float dx = direction ? direction[0] : 0.f, dy = direction ? direction[1] : 0.f, dz = direction ? direction[2] : 1.f;
    CU(launch_gen_rays(scene_of(ctx), kind, seed, pass, dimx, dimy, face, dx, dy, dz, dO, dD, ctx->stream));
    CU(cudaMemcpyAsync(origins, dO, nr * 12, cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaMemcpyAsync(dirs, dD, nr * 12, cudaMemcpyDeviceToHost, ctx->stream));
    return sync_and_status(ctx);
}

int hrt_get_bvh(hrt_context *ctx, uint64_t *codes, uint32_t *perm, uint32_t *nodes) {
    if (!ctx) return HRT_EINVAL;
    int r = check_built(ctx);
    if (r) return r;
    size_t n = (size_t)ctx->n, ni = (size_t)std::max(ctx->n - 1, 1);
    if (n == 0) return HRT_OK;
    if (codes) CU(cudaMemcpy(codes, ctx->codes.p, n * 8, cudaMemcpyDeviceToHost));
    if (perm) CU(cudaMemcpy(perm, ctx->perm.p, n * 4, cudaMemcpyDeviceToHost));
    if (nodes) CU(cudaMemcpy(nodes, ctx->nodes.p, ni * 64, cudaMemcpyDeviceToHost));
    return HRT_OK;
}

void hrt_source_rotation(const float rotation[3], float out[9]) { rotation3(rotation, out); }

int hrt_set_measure(hrt_context *ctx, int flags) {
    if (!ctx) return HRT_EINVAL;
    CU(cudaSetDevice(ctx->device));
    CU(ctx->visits.ensure(ctx->stream, 2 * sizeof(unsigned long long)));
    CU(cudaStreamSynchronize(ctx->stream));
    collect_timings(ctx);
    CU(cudaMemsetAsync(ctx->visits.p, 0, 2 * sizeof(unsigned long long), ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    for (double &m : ctx->meas) m = 0.0;
    ctx->measure = flags;
    return HRT_OK;
}

int hrt_get_measure(hrt_context *ctx, double *out, int count) {
    if (!ctx || !out) return HRT_EINVAL;
    CU(cudaStreamSynchronize(ctx->stream));
    collect_timings(ctx);
    unsigned long long v[2] = {0, 0};
    if (ctx->visits.p) CU(cudaMemcpy(v, ctx->visits.p, sizeof v, cudaMemcpyDeviceToHost));
    ctx->meas[4] = (double)v[0];
    ctx->meas[5] = (double)v[1];
    for (int i = 0; i < count && i < 10; ++i) out[i] = ctx->meas[i];
    return HRT_OK;
}

}  // extern "C"
