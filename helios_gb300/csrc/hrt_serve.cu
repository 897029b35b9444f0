// hrt_serve.cu -- continuous-batching server for radiation solves (host C++ runtime).
//
// Requests name a registered scene and the band set / sun / ray counts of one
// runBand.  A dispatcher thread admits requests in arrival order as soon as
//   (1) their arrival time has passed,
//   (2) the scene's device context is not running another solve, and
//   (3) the scene is resident or fits in the HBM budget (least-recently-used idle
//       scenes are evicted to make room),
// and hands them to a pool of worker threads.  Every resident scene owns an
// hrt_context (BVH, radiation buffers, its own CUDA stream), so solves of
// different scenes run concurrently and overlap on the GPU; a new request for an
// already-resident scene skips the geometry upload and BVH build.
//
// Batching: when a scene's turn comes, every arrived request for that scene with the
// same band set, ray counts, depth and seed joins the batch (up to kMaxChannels
// channels).  A batch of one runs hrt_run_band; a larger batch runs hrt_run_sweep, one
// channel per (request, band): the direct pass is traced per request sun, the diffuse
// and scattering passes once for the whole batch.  Each channel is the solve its
// request would get alone (same Philox streams), so a result depends only on the
// request -- the same alone as in the mix, up to the order of FP64 sums.
//
// Across scenes: the small batches that one dispatch scan admits (different scenes, each
// below kGroupRays traced rays) form one work item, solved by hrt_run_sweep_multi: every
// scene's direct pass and bookkeeping in one captured graph, and each diffuse or scattering
// pass of all of them in one persistent launch (a lone request is a one-sun sweep, which is
// its runBand).  HRT_SERVE_GROUP=0 turns this off.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <iterator>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/hrt.h"

namespace {

using clock_t_ = std::chrono::steady_clock;

struct Scene {
    uint32_t id = 0;
    int32_t n = 0;
    std::vector<float> T;
    std::vector<uint32_t> type;
    std::vector<int8_t> twosided;
    int32_t nbands = 0;
    std::vector<float> rho, tau;  // [n*nbands], one source
    // device state
    hrt_context *ctx = nullptr;
    cudaStream_t stream = nullptr;  // priority stream of this scene's solves
    bool busy = false;
    size_t bytes = 0;
    uint64_t last_use = 0;
};

constexpr int kMaxChannels = 256;  // hrt_run_sweep's channel limit
constexpr uint32_t kRayBudget = 32; // rays per thread before a trace block retires (GPU sharing)
// Batches above this many traced rays run one at a time: interleaved at block granularity,
// several large scenes evict each other's BVH nodes from L1/L2 and the GPU's ray rate
// drops; small batches still run beside them (higher stream priority).
constexpr double kLargeRays = 2e8;
constexpr int kMaxBatch = 64;      // requests per batch
// Batches of at most this many traced rays are grouped across scenes (small solves, where
// per-launch and per-graph overheads weigh most), at most kMaxGroup scenes per group.
constexpr double kGroupRays = 5e7;
constexpr int kMaxGroup = 16;

bool group_enabled() {
    static const bool on = [] {  // initialised once, thread-safe
        const char *e = std::getenv("HRT_SERVE_GROUP");
        return !(e && e[0] == '0');
    }();
    return on;
}

struct Request {
    uint64_t id = 0;
    uint32_t scene = 0;
    double arrival = 0.0;
    std::vector<uint8_t> band_launch;
    float sun[3] = {0, 0, 1};
    std::vector<float> source_flux, diffuse_flux;
    int32_t direct_rays = 100, diffuse_rays = 100, depth = 0;
    uint32_t seed = 0;
    bool keep = false;
    // outcome
    double t_admit = 0.0, t_done = 0.0;
    int status = 1;  // 1 pending, 0 ok, <0 error
    uint64_t rays = 0;
    double checksum = 0.0;
    std::vector<float> flux;
};

// Device bytes of a resident scene solved with Bl bands (records, binary and 4-wide BVH,
// origins, transforms, areas, radiation buffers, BVH scratch).
size_t footprint(int32_t n, int32_t Bl) {
    size_t nn = (size_t)std::max(n, 1);
    return nn * (64 + 64 + 64 + 64 + 64 + 8 + 1) + nn * (size_t)std::max(Bl, 1) * (7 * 8 + 3 * 4) + nn * 200 +
           (8u << 20);
}

}  // namespace

struct hrt_server {
    int device = 0;
    size_t budget = 0, used = 0;
    std::mutex mu;
    std::condition_variable cv_dispatch, cv_work, cv_done;
    std::map<uint32_t, std::unique_ptr<Scene>> scenes;
    std::deque<Request *> arrivals;   // sorted by arrival time when started
    // admitted work, waiting for a worker: one batch, or small batches of different scenes
    std::deque<std::vector<std::vector<Request *>>> ready;
    size_t groups = 0, grouped_batches = 0;
    std::map<uint64_t, std::unique_ptr<Request>> requests;
    std::vector<std::thread> workers;
    std::thread dispatcher;
    bool started = false, stopping = false;
    size_t outstanding = 0, evictions = 0, builds = 0, batches = 0, batched_requests = 0;
    std::mutex large;  // held by the one large batch in flight
    clock_t_::time_point t0;
    uint64_t tick = 0;
    std::string err;

    double now() const { return std::chrono::duration<double>(clock_t_::now() - t0).count(); }
};

namespace {

bool ensure_resident(hrt_server *s, Scene *sc, int32_t Bl, std::string &err) {
    // caller holds s->mu; scene is not busy
    size_t need = footprint(sc->n, Bl);
    if (sc->ctx && need <= sc->bytes) return true;
    size_t extra = need - (sc->ctx ? sc->bytes : 0);
    while (s->used + extra > s->budget) {
        Scene *victim = nullptr;
        for (auto &kv : s->scenes) {
            Scene *c = kv.second.get();
            if (c != sc && c->ctx && !c->busy && (!victim || c->last_use < victim->last_use)) victim = c;
        }
        if (!victim) return false;  // wait for a busy scene to finish
        hrt_destroy(victim->ctx);
        victim->ctx = nullptr;
        if (victim->stream) {
            cudaSetDevice(s->device);
            cudaStreamDestroy(victim->stream);
            victim->stream = nullptr;
        }
        s->used -= victim->bytes;
        victim->bytes = 0;
        ++s->evictions;
    }
    s->used += extra;
    sc->bytes = need;
    (void)err;
    return true;
}

bool same_batch(const Request *a, const Request *b) {
    return a->scene == b->scene && a->band_launch == b->band_launch && a->direct_rays == b->direct_rays &&
           a->diffuse_rays == b->diffuse_rays && a->depth == b->depth && a->seed == b->seed;
}

// One request alone: a full runBand.
int solve_one(Scene *sc, Request *r, int Bl) {
    hrt_source src{};
    src.type = 0;
    for (int k = 0; k < 3; ++k) src.position[k] = r->sun[k];
    std::vector<int32_t> dr(Bl, r->direct_rays), fr(Bl, r->diffuse_rays), dp(Bl, r->depth);
    std::vector<uint8_t> em(Bl, 0);
    hrt_band_solve b{};
    b.nbands_global = sc->nbands;
    b.band_launch = r->band_launch.data();
    b.nsources = 1;
    b.sources = &src;
    b.source_flux = r->source_flux.data();
    b.diffuse_flux = r->diffuse_flux.data();
    b.direct_rays = dr.data();
    b.diffuse_rays = fr.data();
    b.scattering_depth = dp.data();
    b.emission = em.data();
    b.seed = r->seed;
    std::vector<float> flux((size_t)sc->n * Bl);
    int rc = hrt_run_band(sc->ctx, &b, flux.data());
    if (rc != HRT_OK) return rc;
    uint64_t st[2] = {0, 0};
    hrt_last_stats(sc->ctx, st, 2);
    r->rays = st[0];
    double sum = 0.0;
    for (float f : flux) sum += f;
    r->checksum = sum;
    if (r->keep) r->flux.swap(flux);
    return HRT_OK;
}

int launched_bands(const Request *r) {
    int Bl = 0;
    for (uint8_t f : r->band_launch) Bl += f ? 1 : 0;
    return Bl;
}

// Traced rays of a batch (direct rays per request, diffuse passes shared).
double batch_rays(const Scene *sc, const std::vector<Request *> &batch) {
    const Request *r0 = batch[0];
    const double side = std::ceil(std::sqrt((double)r0->diffuse_rays));
    return (double)sc->n * ((double)r0->direct_rays * (double)batch.size() + 2.0 * side * side * (1.0 + (double)r0->depth));
}

// The sweep of a batch of compatible requests: channel c = request * Bl + band.
struct SweepInput {
    std::vector<float> rho, tau, sun, dflux, sflux, out;
    hrt_sweep w{};
    int Bl = 0;
};

void make_sweep(const Scene *sc, const std::vector<Request *> &batch, SweepInput *in) {
    const int Bl = launched_bands(batch[0]);
    const int nr = (int)batch.size(), C = nr * Bl;
    const size_t n = (size_t)sc->n;
    std::vector<int> cols;
    for (int b = 0; b < sc->nbands; ++b)
        if (batch[0]->band_launch[b]) cols.push_back(b);
    in->Bl = Bl;
    in->rho.assign(n * Bl, 0.f);
    in->tau.assign(n * Bl, 0.f);
    in->sun.assign(3 * (size_t)nr, 0.f);
    in->dflux.assign(C, 0.f);
    in->sflux.assign(C, 0.f);
    in->out.assign(n * C, 0.f);
    for (size_t p = 0; p < n; ++p)
        for (int b = 0; b < Bl; ++b) {
            in->rho[p * Bl + b] = sc->rho[p * sc->nbands + cols[b]];
            in->tau[p * Bl + b] = sc->tau[p * sc->nbands + cols[b]];
        }
    for (int i = 0; i < nr; ++i) {
        for (int k = 0; k < 3; ++k) in->sun[3 * i + k] = batch[i]->sun[k];
        for (int b = 0; b < Bl; ++b) {
            in->dflux[i * Bl + b] = batch[i]->source_flux[b];
            in->sflux[i * Bl + b] = batch[i]->diffuse_flux[b];
        }
    }
    hrt_sweep &w = in->w;
    w = hrt_sweep{};
    w.nsun = nr;
    w.sun_dir = in->sun.data();
    w.nbands = Bl;
    w.direct_flux = in->dflux.data();
    w.diffuse_flux = in->sflux.data();
    w.rho = in->rho.data();
    w.tau = in->tau.data();
    w.direct_rays = batch[0]->direct_rays;
    w.diffuse_rays = batch[0]->diffuse_rays;
    w.scattering_depth = batch[0]->depth;
    w.seed = batch[0]->seed;
}

// Results of a solved sweep back to its requests; rays of the batch shared evenly.
void take_results(const Scene *sc, const std::vector<Request *> &batch, const SweepInput &in, uint64_t rays) {
    const int nr = (int)batch.size(), Bl = in.Bl, C = nr * Bl;
    const size_t n = (size_t)sc->n;
    const std::vector<float> &out = in.out;
    for (int i = 0; i < nr; ++i) {
        Request *r = batch[i];
        r->rays = rays / (uint64_t)nr;
        std::vector<float> flux(n * Bl);
        double sum = 0.0;
        for (size_t p = 0; p < n; ++p)
            for (int b = 0; b < Bl; ++b) {
                const float v = out[p * C + (size_t)i * Bl + b];
                flux[p * Bl + b] = v;
                sum += v;
            }
        r->checksum = sum;
        if (r->keep) r->flux.swap(flux);
    }
}

int solve_batch(Scene *sc, const std::vector<Request *> &batch) {
    SweepInput in;
    make_sweep(sc, batch, &in);
    int rc = hrt_run_sweep(sc->ctx, &in.w, in.out.data());
    if (rc != HRT_OK) return rc;
    uint64_t st[2] = {0, 0};
    hrt_last_stats(sc->ctx, st, 2);
    take_results(sc, batch, in, st[0]);
    return HRT_OK;
}

// Small batches of different scenes: one multi-scene sweep.
int solve_group(const std::vector<Scene *> &scs, const std::vector<std::vector<Request *>> &batches) {
    const size_t k = scs.size();
    std::vector<SweepInput> in(k);
    std::vector<hrt_context *> ctxs(k);
    std::vector<hrt_sweep> sweeps(k);
    std::vector<float *> outs(k);
    for (size_t i = 0; i < k; ++i) {
        make_sweep(scs[i], batches[i], &in[i]);
        ctxs[i] = scs[i]->ctx;
        sweeps[i] = in[i].w;
        outs[i] = in[i].out.data();
    }
    int rc = hrt_run_sweep_multi(ctxs.data(), sweeps.data(), (int32_t)k, outs.data());
    if (rc != HRT_OK) return rc;
    for (size_t i = 0; i < k; ++i) {
        uint64_t st[2] = {0, 0};
        hrt_last_stats(scs[i]->ctx, st, 2);
        take_results(scs[i], batches[i], in[i], st[0]);
    }
    return HRT_OK;
}

// Device context of a scene: created, geometry uploaded, BVH built and materials set the
// first time the scene is solved (or after an eviction).
int prepare_scene(hrt_server *s, Scene *sc) {
    if (sc->ctx) return HRT_OK;
    int rc = hrt_create(&sc->ctx, s->device);
    if (rc == HRT_OK) {
        // Smaller scenes get higher stream priority and every trace block retires after
        // kRayBudget rays per thread, so a small solve's blocks start as soon as SMs free up
        // instead of waiting for a large solve to end.
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        double f = (std::log10((double)std::max(sc->n, 1)) - 3.0) / 3.5;  // 1e3 .. 3e6 prims
        f = std::min(1.0, std::max(0.0, f));
        const int prio = greatest + (int)std::lround(f * (double)(least - greatest));
        if (cudaStreamCreateWithPriority(&sc->stream, cudaStreamNonBlocking, prio) == cudaSuccess)
            rc = hrt_set_stream(sc->ctx, sc->stream);
        if (rc == HRT_OK) rc = hrt_set_ray_budget(sc->ctx, kRayBudget);
        // fixed default kernels: timing trials per scene would cost more than they save
        if (rc == HRT_OK) rc = hrt_set_tuning(sc->ctx, 0);
    }
    if (rc == HRT_OK) {
        hrt_geometry g{};
        g.n = sc->n;
        g.transform = sc->T.data();
        g.type = sc->type.data();
        g.twosided = sc->twosided.data();
        rc = hrt_update_geometry(sc->ctx, &g);
        if (rc == HRT_OK) rc = hrt_build_accel(sc->ctx);
        if (rc == HRT_OK) rc = hrt_update_materials(sc->ctx, 1, sc->n, sc->nbands, sc->rho.data(), sc->tau.data());
        std::lock_guard<std::mutex> lk(s->mu);
        ++s->builds;
    }
    return rc;
}

void worker_loop(hrt_server *s) {
    for (;;) {
        std::vector<std::vector<Request *>> item;
        std::vector<Scene *> scs;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stopping || !s->ready.empty(); });
            if (s->stopping && s->ready.empty()) return;
            item.swap(s->ready.front());
            s->ready.pop_front();
            for (const auto &b : item) scs.push_back(s->scenes[b[0]->scene].get());
        }
        int rc = HRT_OK;
        for (Scene *sc : scs)
            if (rc == HRT_OK) rc = prepare_scene(s, sc);
        if (rc == HRT_OK && item.size() > 1) {
            rc = solve_group(scs, item);
        } else if (rc == HRT_OK) {
            Scene *sc = scs[0];
            std::vector<Request *> &batch = item[0];
            const int Bl = launched_bands(batch[0]);
            std::unique_lock<std::mutex> gate(s->large, std::defer_lock);
            if (batch_rays(sc, batch) > kLargeRays) {
                gate.lock();
                // requests of this scene that arrived while the batch waited for the GPU
                // join it (the scene is busy, so they would otherwise wait for the next batch)
                std::lock_guard<std::mutex> lk(s->mu);
                const double t = s->now();
                for (auto it = s->arrivals.begin(); it != s->arrivals.end() && (int)batch.size() < kMaxBatch &&
                                                    (int)(batch.size() + 1) * Bl <= kMaxChannels;) {
                    Request *q = *it;
                    if (q->arrival > t) break;
                    if (same_batch(batch[0], q)) {
                        q->t_admit = t;
                        batch.push_back(q);
                        ++s->batched_requests;
                        it = s->arrivals.erase(it);  // erase returns a valid iterator to the next one
                    } else {
                        ++it;
                    }
                }
            }
            rc = batch.size() == 1 ? solve_one(sc, batch[0], Bl) : solve_batch(sc, batch);
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            const double t = s->now();
            for (const auto &batch : item)
                for (Request *r : batch) {
                    r->t_done = t;
                    r->status = rc;
                    --s->outstanding;
                }
            if (rc != HRT_OK) {
                for (Scene *sc : scs)
                    if (sc->ctx && s->err.empty()) s->err = hrt_last_error(sc->ctx);
            }
            for (Scene *sc : scs) {
                sc->busy = false;
                sc->last_use = ++s->tick;
            }
        }
        s->cv_dispatch.notify_all();
        s->cv_done.notify_all();
    }
}

void dispatch_loop(hrt_server *s) {
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        if (s->stopping) return;
        if (s->arrivals.empty()) {
            s->cv_dispatch.wait(lk);
            continue;
        }
        double t = s->now();
        bool admitted = false;
        double next_arrival = -1.0;
        std::vector<std::vector<Request *>> small;  // this scan's small batches (different scenes)
        // scan requests that have arrived, in arrival order; admit every one whose scene
        // is idle and fits (continuous batching: later requests may pass a blocked one)
        for (auto it = s->arrivals.begin(); it != s->arrivals.end();) {
            Request *r = *it;
            if (r->arrival > t) {
                next_arrival = r->arrival;
                break;
            }
            Scene *sc = s->scenes[r->scene].get();
            int Bl = 0;
            for (uint8_t f : r->band_launch) Bl += f ? 1 : 0;
            std::string err;
            if (!sc->busy && ensure_resident(s, sc, Bl, err)) {
                sc->busy = true;
                r->t_admit = t;
                std::vector<Request *> batch{r};
                // later arrived requests of the same scene and solve settings join the batch
                for (auto jt = std::next(it); jt != s->arrivals.end() && (int)batch.size() < kMaxBatch &&
                                              (int)(batch.size() + 1) * Bl <= kMaxChannels;
                     ++jt) {
                    Request *q = *jt;
                    if (q->arrival > t) break;
                    if (same_batch(r, q)) {
                        q->t_admit = t;
                        batch.push_back(q);
                    }
                }
                // erasing from a deque invalidates its iterators: remove the batch, rescan
                s->arrivals.erase(std::remove_if(s->arrivals.begin(), s->arrivals.end(),
                                                 [&](const Request *x) {
                                                     return std::find(batch.begin(), batch.end(), x) != batch.end();
                                                 }),
                                  s->arrivals.end());
                ++s->batches;
                s->batched_requests += batch.size();
                if (group_enabled() && batch_rays(sc, batch) <= kGroupRays) {
                    small.push_back(std::move(batch));
                    if ((int)small.size() == kMaxGroup) {
                        s->ready.push_back(std::move(small));
                        small.clear();
                    }
                } else {
                    s->ready.push_back({std::move(batch)});
                }
                admitted = true;
                it = s->arrivals.begin();
            } else {
                ++it;
            }
        }
        if (!small.empty()) {
            if (small.size() > 1) {
                ++s->groups;
                s->grouped_batches += small.size();
            }
            s->ready.push_back(std::move(small));
        }
        if (admitted) {
            s->cv_work.notify_all();
            continue;
        }
        if (next_arrival >= 0.0) {
            auto wake = s->t0 + std::chrono::duration_cast<clock_t_::duration>(std::chrono::duration<double>(next_arrival));
            s->cv_dispatch.wait_until(lk, wake);
        } else {
            s->cv_dispatch.wait(lk);  // arrived requests are blocked on busy scenes / memory
        }
    }
}

}  // namespace

extern "C" {

int hrt_server_create(hrt_server **out, int device, int workers, size_t hbm_budget_bytes) {
    if (!out || workers < 1 || workers > 256 || hbm_budget_bytes == 0) return HRT_EINVAL;
    hrt_server *s = new hrt_server();
    s->device = device;
    s->budget = hbm_budget_bytes;
    s->t0 = clock_t_::now();
    for (int i = 0; i < workers; ++i) s->workers.emplace_back(worker_loop, s);
    *out = s;
    return HRT_OK;
}

int hrt_server_add_scene(hrt_server *s, uint32_t scene_id, const hrt_geometry *g, int32_t nbands_global,
                         const float *rho, const float *tau) {
    if (!s || !g || g->n < 1 || nbands_global < 1 || !rho || !tau || !g->transform || !g->type || !g->twosided)
        return HRT_EINVAL;
    if (g->nbbox != 0) return HRT_EUNSUPPORTED;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->started) return HRT_EINVAL;
    auto sc = std::make_unique<Scene>();
    sc->id = scene_id;
    sc->n = g->n;
    sc->T.assign(g->transform, g->transform + 16 * (size_t)g->n);
    sc->type.assign(g->type, g->type + g->n);
    sc->twosided.assign(g->twosided, g->twosided + g->n);
    sc->nbands = nbands_global;
    sc->rho.assign(rho, rho + (size_t)g->n * nbands_global);
    sc->tau.assign(tau, tau + (size_t)g->n * nbands_global);
    s->scenes[scene_id] = std::move(sc);
    return HRT_OK;
}

int hrt_server_submit(hrt_server *s, const hrt_serve_request *q) {
    if (!s || !q || !q->band_launch) return HRT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto sit = s->scenes.find(q->scene_id);
    if (sit == s->scenes.end()) return HRT_EINVAL;
    Scene *sc = sit->second.get();
    auto r = std::make_unique<Request>();
    r->id = q->request_id;
    r->scene = q->scene_id;
    r->arrival = q->arrival_s;
    r->band_launch.assign(q->band_launch, q->band_launch + sc->nbands);
    int Bl = 0;
    for (uint8_t f : r->band_launch) Bl += f ? 1 : 0;
    if (Bl < 1 || !q->source_flux || !q->diffuse_flux) return HRT_EINVAL;
    if (footprint(sc->n, Bl) > s->budget) return HRT_ENOMEM;  // could never be admitted
    for (int k = 0; k < 3; ++k) r->sun[k] = q->sun_dir[k];
    r->source_flux.assign(q->source_flux, q->source_flux + Bl);
    r->diffuse_flux.assign(q->diffuse_flux, q->diffuse_flux + Bl);
    r->direct_rays = q->direct_rays;
    r->diffuse_rays = q->diffuse_rays;
    r->depth = q->scattering_depth;
    r->seed = q->seed;
    r->keep = q->keep_result != 0;
    Request *raw = r.get();
    s->requests[r->id] = std::move(r);
    // keep arrivals sorted
    auto pos = std::upper_bound(s->arrivals.begin(), s->arrivals.end(), raw,
                                [](const Request *a, const Request *b) { return a->arrival < b->arrival; });
    s->arrivals.insert(pos, raw);
    ++s->outstanding;
    if (s->started) s->cv_dispatch.notify_all();
    return HRT_OK;
}

int hrt_server_start(hrt_server *s) {
    if (!s) return HRT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->started) return HRT_OK;
    s->started = true;
    s->t0 = clock_t_::now();
    s->dispatcher = std::thread(dispatch_loop, s);
    return HRT_OK;
}

int hrt_server_wait(hrt_server *s) {
    if (!s) return HRT_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->outstanding == 0; });
    for (auto &kv : s->requests)
        if (kv.second->status < 0) return kv.second->status;
    return HRT_OK;
}

int hrt_server_result(hrt_server *s, uint64_t request_id, float *flux_out, size_t count, double *timing,
                      double *checksum, uint64_t *rays) {
    if (!s) return HRT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return HRT_EINVAL;
    Request *r = it->second.get();
    if (r->status == 1) return HRT_EINVAL;
    if (timing) {
        timing[0] = r->arrival;
        timing[1] = r->t_admit;
        timing[2] = r->t_done;
    }
    if (checksum) *checksum = r->checksum;
    if (rays) *rays = r->rays;
    if (flux_out && count) {
        if (r->flux.size() != count) return HRT_EINVAL;
        std::memcpy(flux_out, r->flux.data(), count * sizeof(float));
    }
    return r->status;
}

int hrt_server_stats(hrt_server *s, double *out, int count) {
    if (!s || !out) return HRT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    double v[8] = {(double)s->builds,  (double)s->evictions, (double)s->used,           (double)s->budget,
                   (double)s->batches, (double)s->batched_requests, (double)s->groups, (double)s->grouped_batches};
    for (int i = 0; i < count && i < 8; ++i) out[i] = v[i];
    return HRT_OK;
}

int hrt_server_destroy(hrt_server *s) {
    if (!s) return HRT_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_dispatch.notify_all();
    s->cv_work.notify_all();
    if (s->dispatcher.joinable()) s->dispatcher.join();
    for (auto &t : s->workers) t.join();
    for (auto &kv : s->scenes) {
        if (kv.second->ctx) hrt_destroy(kv.second->ctx);
        if (kv.second->stream) {
            cudaSetDevice(s->device);
            cudaStreamDestroy(kv.second->stream);
        }
    }
    delete s;
    return HRT_OK;
}

}  // extern "C"
