// hrt_static.cu -- BVH build that allocates nothing.
//
// Some callers cannot call cudaMalloc: code that hands every byte of device
// memory out of its own arena or framework allocator, and latency-critical loops
// where a cudaMalloc/cudaFree would synchronise the whole device.  For them
// hrt_build_accel_static() builds the same LBVH as hrt_build_accel() from
// caller-owned device buffers into caller-owned device buffers.  Its scratch
// (sort buffers, boxes, parent links, arrival counters, the error word) lives in
// one file-scope static device array below, sized for at most
// HRT_STATIC_MAX_PRIMS primitives; every GPU that loads this library holds that
// array (about 5.6 MB) until the process exits.
//
// The first call on each device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it per device index;
// make that first call before any stream capture.  A cudaDeviceReset of a device
// invalidates its cached address: reload the library after one.
//
// Each call ends by reading the error word back on the caller's stream and waiting
// for that stream; it never waits for the device or for other streams.
//
// All calls share the array and it keeps the last call's contents; the parts
// that must start at zero (arrival counters, parent links, the error word) are
// cleared on every call.  Two calls whose work overlaps on the GPU (different
// streams, or different host threads) race on the array and corrupt each other.
#include <mutex>

#include "../../include/hrt.h"
#include "hrt_internal.h"

using namespace hrt;

namespace {

constexpr int kMaxPrims = HRT_STATIC_MAX_PRIMS;
constexpr size_t kStatusBytes = 256;  // error word, kept apart from the build scratch
constexpr size_t kScratchBytes = kStatusBytes + bvh_scratch_bytes_c(kMaxPrims);

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_scratch on the current device.  In host code the symbol
// g_scratch names a host-side stand-in, not device memory, so the address is
// looked up once per device (with that device current) and cached.
int scratch_address(void **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return HRT_ECUDA;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return HRT_ECUDA;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return HRT_OK;
}

}  // namespace

extern "C" int hrt_build_accel_static(const float *d_transform, const uint32_t *d_type, int32_t n,
                                      void *d_records, void *d_origins, void *d_nodes, uint64_t *d_codes,
                                      uint32_t *d_perm, void *stream) {
    if (n < 1 || n > kMaxPrims) return HRT_EINVAL;
    if (!d_transform || !d_type || !d_records || !d_origins || !d_nodes || !d_codes || !d_perm) return HRT_EINVAL;
    void *base = nullptr;
    int r = scratch_address(&base);
    if (r != HRT_OK) return r;
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *status = (uint32_t *)base;
    if (cudaMemsetAsync(status, 0, sizeof(uint32_t), s) != cudaSuccess) return HRT_ECUDA;
    BvhBuffers b;
    bvh_carve(b, (char *)base + kStatusBytes, n);
    b.rec = (float4 *)d_records;
    b.rgen = (float4 *)d_origins;
    b.nodes = (float4 *)d_nodes;
    b.codes = d_codes;
    b.perm = d_perm;
    b.status = status;
    if (bvh_build(d_transform, d_type, nullptr, n, b, s) != cudaSuccess) return HRT_ECUDA;
    uint32_t st = 0;
    if (cudaMemcpyAsync(&st, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess) return HRT_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return HRT_ECUDA;
    return st ? HRT_EDEVICE : HRT_OK;
}
