// ref_raycast.cpp -- C entry points over the REFERENCE's own CPU ray caster (test
// infrastructure only; built by oracle/ref.mk into oracle/_ref/ next to the reference's
// core and CollisionDetection sources, compiled unchanged from the reference tree).
//
// The scene is loaded into a helios::Context primitive by primitive: patches through
// Context::addPatch() (core/src/Context_primitive.cpp:20) and triangles through
// Context::addTriangle(), then each primitive's transform is set to the caller's
// (Context::setPrimitiveTransformationMatrix, core/src/Context.cpp:3249), so that the
// reference derives its vertices from the same FP32 matrices the oracle and the GPU read
// (Patch/Triangle::getVertices, core/src/Context_primitive.cpp:891-915).  Rays go through
// CollisionDetection::castRaysSoA (plugins/collisiondetection/src/
// CollisionDetection_RayTracing.cpp:551-680): its own BVH, its own triangle and patch
// tests (CollisionDetection_RayTracing.cpp:1555-1630), closest hit, t > 1e-6.
#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include "CollisionDetection.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct RefScene {
    helios::Context ctx;
    std::unique_ptr<CollisionDetection> cd;
    std::vector<int64_t> index_of_uuid;  // Context UUID -> caller's primitive index
};

thread_local std::string g_err;

helios::vec3 apply(const float *T, float x, float y) {
    // same sums as Patch/Triangle::getVertices (z = 0 in the canonical shapes)
    return helios::make_vec3(T[0] * x + T[1] * y + T[2] * 0.f + T[3], T[4] * x + T[5] * y + T[6] * 0.f + T[7],
                             T[8] * x + T[9] * y + T[10] * 0.f + T[11]);
}

}  // namespace

extern "C" {

const char *ref_last_error(void) { return g_err.c_str(); }

// n primitives of type 0 (patch) or 1 (triangle) with row-major 4x4 transforms T16 [n*16].
// Returns a handle, or NULL with ref_last_error() set.
void *ref_scene_create(int32_t n, const float *T16, const uint32_t *type) {
    try {
        auto *s = new RefScene();
        for (int32_t i = 0; i < n; ++i) {
            const float *T = T16 + 16 * (size_t)i;
            uint32_t uuid;
            if (type[i] == 0) {
                uuid = s->ctx.addPatch();
            } else if (type[i] == 1) {
                uuid = s->ctx.addTriangle(apply(T, 0.f, 0.f), apply(T, 0.f, 1.f), apply(T, 1.f, 1.f));
            } else {
                delete s;
                g_err = "only patches (0) and triangles (1) are supported";
                return nullptr;
            }
            float M[16];
            std::memcpy(M, T, sizeof M);
            s->ctx.setPrimitiveTransformationMatrix(uuid, M);
            if (s->index_of_uuid.size() <= uuid) s->index_of_uuid.resize((size_t)uuid + 1, -1);
            s->index_of_uuid[uuid] = i;
        }
        s->cd = std::make_unique<CollisionDetection>(&s->ctx);
        s->cd->disableMessages();
        s->cd->buildBVH();
        return s;
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

// Closest hits of nrays rays (origins o, unit directions d, [nrays*3]): out_index = the
// caller's primitive index or -1 (miss), out_t = hit distance.  threads 0: OpenMP default.
int ref_cast_rays(void *h, int64_t nrays, const float *o, const float *d, float max_distance, int64_t *out_index,
                  float *out_t, int threads) {
    try {
        auto *s = static_cast<RefScene *>(h);
#ifdef _OPENMP
        if (threads > 0) omp_set_num_threads(threads);
#else
        (void)threads;
#endif
        std::vector<helios::vec3> org((size_t)nrays), dir((size_t)nrays), nrm((size_t)nrays);
        for (int64_t i = 0; i < nrays; ++i) {
            org[i] = helios::make_vec3(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
            dir[i] = helios::make_vec3(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
        }
        std::vector<uint> uuid((size_t)nrays);
        s->cd->castRaysSoA(org.data(), dir.data(), (size_t)nrays, max_distance, out_t, nrm.data(), uuid.data());
        for (int64_t i = 0; i < nrays; ++i) {
            const uint u = uuid[i];
            out_index[i] = (u == 0xFFFFFFFFu || u >= s->index_of_uuid.size()) ? -1 : s->index_of_uuid[u];
        }
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

void ref_scene_free(void *h) { delete static_cast<RefScene *>(h); }

}  // extern "C"
