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
// already-resident scene skips the geometry upload and BVH build.  Each solve is
// a full hrt_run_band, so a request's result depends only on its scene, band set,
// sun, ray counts and seed -- the same alone as in the mix.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

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
    bool busy = false;
    size_t bytes = 0;
    uint64_t last_use = 0;
};

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

// Device bytes of a resident scene solved with Bl bands (records, BVH, origins,
// transforms, radiation buffers, BVH scratch).
size_t footprint(int32_t n, int32_t Bl) {
    size_t nn = (size_t)std::max(n, 1);
    return nn * (64 + 64 + 64 + 64 + 1) + nn * (size_t)std::max(Bl, 1) * (7 * 8 + 3 * 4) + nn * 200 + (8u << 20);
}

}  // namespace

struct hrt_server {
    int device = 0;
    size_t budget = 0, used = 0;
    std::mutex mu;
    std::condition_variable cv_dispatch, cv_work, cv_done;
    std::map<uint32_t, std::unique_ptr<Scene>> scenes;
    std::deque<Request *> arrivals;   // sorted by arrival time when started
    std::deque<Request *> ready;      // admitted, waiting for a worker
    std::map<uint64_t, std::unique_ptr<Request>> requests;
    std::vector<std::thread> workers;
    std::thread dispatcher;
    bool started = false, stopping = false;
    size_t outstanding = 0, evictions = 0, builds = 0;
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
        s->used -= victim->bytes;
        victim->bytes = 0;
        ++s->evictions;
    }
    s->used += extra;
    sc->bytes = need;
    (void)err;
    return true;
}

void worker_loop(hrt_server *s) {
    for (;;) {
        Request *r = nullptr;
        Scene *sc = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stopping || !s->ready.empty(); });
            if (s->stopping && s->ready.empty()) return;
            r = s->ready.front();
            s->ready.pop_front();
            sc = s->scenes[r->scene].get();
        }
        int rc = HRT_OK;
        if (!sc->ctx) {
            rc = hrt_create(&sc->ctx, s->device);
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
        }
        int Bl = 0;
        for (uint8_t f : r->band_launch) Bl += f ? 1 : 0;
        if (rc == HRT_OK) {
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
            rc = hrt_run_band(sc->ctx, &b, flux.data());
            if (rc == HRT_OK) {
                uint64_t st[2] = {0, 0};
                hrt_last_stats(sc->ctx, st, 2);
                r->rays = st[0];
                double sum = 0.0;
                for (float f : flux) sum += f;
                r->checksum = sum;
                if (r->keep) r->flux.swap(flux);
            }
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            r->t_done = s->now();
            r->status = rc;
            if (rc != HRT_OK && sc->ctx) s->err = hrt_last_error(sc->ctx);
            sc->busy = false;
            sc->last_use = ++s->tick;
            --s->outstanding;
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
                s->ready.push_back(r);
                it = s->arrivals.erase(it);
                admitted = true;
            } else {
                ++it;
            }
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
    double v[4] = {(double)s->builds, (double)s->evictions, (double)s->used, (double)s->budget};
    for (int i = 0; i < count && i < 4; ++i) out[i] = v[i];
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
    for (auto &kv : s->scenes)
        if (kv.second->ctx) hrt_destroy(kv.second->ctx);
    delete s;
    return HRT_OK;
}

}  // extern "C"
