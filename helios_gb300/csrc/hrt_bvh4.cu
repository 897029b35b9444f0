// hrt_bvh4.cu -- compressed 4-wide BVH from a binary BVH (the clustered tree of ploc_build).
//
// The diffuse trace is bound by L1 traffic of node fetches (64 B per visit of a binary
// node).  A 4-wide node with 8-bit child boxes (node format in hrt_device.cuh) is also
// 64 B but covers two tree levels, so a ray fetches about half the node bytes and follows
// half as many dependent loads.  The collapse runs top-down in waves, one thread per node
// of the wave: starting from the two children of a binary node, the internal child with
// the largest surface area is replaced by its two children until there are four (or only
// leaves are left); every internal child gets a new 4-wide node in the next wave.  Child
// sets depend only on the binary tree, so traversal results and visit counts do not depend
// on the order in which atomics hand out node indices.
#include <algorithm>

#include "hrt_device.cuh"
#include "hrt_internal.h"

namespace hrt {

namespace {

constexpr int kThreads4 = 256;

struct Box {
    float lo[3], hi[3];
};

__device__ __forceinline__ void child_box(const float4 *__restrict__ n2, int32_t node, int k, Box *b) {
    const float4 *nd = n2 + 4 * (size_t)node;
    float4 a = nd[0], c = nd[1], d = nd[2];
    if (k == 0) {
        *b = Box{{a.x, a.y, a.z}, {a.w, c.x, c.y}};
    } else {
        *b = Box{{c.z, c.w, d.x}, {d.y, d.z, d.w}};
    }
}

__device__ __forceinline__ float half_area(const Box &b) {
    float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// Smallest step s = 2^(e-127) with p + 255 s >= hi (FP32, as decoded); e in [1, 254].
__device__ __forceinline__ uint32_t pick_exponent(float p, float hi) {
    float x = (hi - p) * (1.0f / 255.0f);
    uint32_t bits = __float_as_uint(x);
    uint32_t e = (bits >> 23) & 0xFFu;
    if (bits & 0x7FFFFFu) e += 1;
    if (e < 1) e = 1;
    while (e < 254 && !(q_decode(p, 255u, q_step(e)) >= hi)) ++e;
    return e;
}

__device__ __forceinline__ uint32_t quant_lo(float p, float v, float s) {
    float f = floorf((v - p) / s);
    int q = f < 0.f ? 0 : (f > 255.f ? 255 : (int)f);
    while (q > 0 && q_decode(p, (uint32_t)q, s) > v) --q;
    return (uint32_t)q;
}

__device__ __forceinline__ uint32_t quant_hi(float p, float v, float s) {
    float f = ceilf((v - p) / s);
    int q = f < 0.f ? 0 : (f > 255.f ? 255 : (int)f);
    while (q < 255 && q_decode(p, (uint32_t)q, s) < v) ++q;
    return (uint32_t)q;
}

// One wave: item i turns binary node in[i].x into 4-wide node in[i].y.
// cap: 4-wide nodes n4 holds; qcap: items the wave queues hold.
__global__ void __launch_bounds__(kThreads4) k_collapse(int n2count, const float4 *__restrict__ n2,
                                                        const int2 *__restrict__ in, int nin, int2 *__restrict__ out,
                                                        unsigned *__restrict__ nout, unsigned *__restrict__ nnodes,
                                                        int cap, int qcap, float4 *__restrict__ n4,
                                                        uint32_t *__restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nin) return;
    const int32_t b = in[i].x, q = in[i].y;
    if (b < 0 || b >= n2count || q < 0 || q >= cap) {
        atomicOr(status, ERR_BOUNDS);
        return;
    }
    int32_t ref[4];
    Box box[4];
    const float4 *nd = n2 + 4 * (size_t)b;
    ref[0] = __float_as_int(nd[3].x);
    ref[1] = __float_as_int(nd[3].y);
    child_box(n2, b, 0, &box[0]);
    child_box(n2, b, 1, &box[1]);
    int cnt = 2;
    while (cnt < 4) {
        int best = -1;
        float ba = -1.f;
        for (int k = 0; k < cnt; ++k) {
            if (ref[k] < 0) continue;  // leaf or empty
            float a = half_area(box[k]);
            if (a > ba) {
                ba = a;
                best = k;
            }
        }
        if (best < 0) break;
        const int32_t c = ref[best];
        if (c >= n2count) {
            atomicOr(status, ERR_BOUNDS);
            return;
        }
        const float4 *cd = n2 + 4 * (size_t)c;
        ref[best] = __float_as_int(cd[3].x);
        ref[cnt] = __float_as_int(cd[3].y);
        child_box(n2, c, 0, &box[best]);
        child_box(n2, c, 1, &box[cnt]);
        ++cnt;
    }
    // node box and steps over the children that exist
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < cnt; ++k) {
        if (ref[k] == kEmptyChild) continue;
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], box[k].lo[a]);
            hi[a] = fmaxf(hi[a], box[k].hi[a]);
        }
    }
    if (!(lo[0] <= hi[0])) {  // no child: cannot happen for a built tree
        for (int a = 0; a < 3; ++a) lo[a] = hi[a] = 0.f;
    }
    float s[3];
    for (int a = 0; a < 3; ++a) s[a] = q_step(pick_exponent(lo[a], hi[a]));
    uint32_t wlo[3] = {0, 0, 0}, whi[3] = {0, 0, 0};
    int32_t outref[4] = {kEmptyChild, kEmptyChild, kEmptyChild, kEmptyChild};
    // The internal children of a node get consecutive indices from one allocation, padded to
    // an even count: every allocation starts on an even index, i.e. on a 128-byte line of two
    // 64-byte nodes, so siblings (which rays tend to visit one after another) share lines.
    int nint = 0;
    for (int k = 0; k < cnt; ++k) nint += ref[k] >= 0 ? 1 : 0;
    unsigned nq0 = 0, slot0 = 0;
    if (nint > 0) {
        nq0 = atomicAdd(nnodes, (unsigned)((nint + 1) & ~1));
        slot0 = atomicAdd(nout, (unsigned)nint);
    }
    int j = 0;
    for (int k = 0; k < 4; ++k) {
        const int32_t c = k < cnt ? ref[k] : kEmptyChild;
        if (c == kEmptyChild) {  // inverted box: lo bytes 255, hi bytes 0
            for (int a = 0; a < 3; ++a) wlo[a] |= 0xFFu << (8 * k);
            continue;
        }
        for (int a = 0; a < 3; ++a) {
            wlo[a] |= quant_lo(lo[a], box[k].lo[a], s[a]) << (8 * k);
            whi[a] |= quant_hi(lo[a], box[k].hi[a], s[a]) << (8 * k);
        }
        if (c < 0) {
            outref[k] = c;  // leaf: ~slot
        } else {
            const unsigned nq = nq0 + (unsigned)j, slot = slot0 + (unsigned)j;
            ++j;
            if ((int)nq >= cap || (int)slot >= qcap) {
                atomicOr(status, ERR_BOUNDS);
                continue;
            }
            outref[k] = (int32_t)nq;
            out[slot] = make_int2(c, (int32_t)nq);
        }
    }
    float4 *o = n4 + 4 * (size_t)q;
    o[0] = make_float4(lo[0], lo[1], lo[2], s[0]);
    o[1] = make_float4(__uint_as_float(wlo[0]), __uint_as_float(wlo[1]), __uint_as_float(wlo[2]),
                       __uint_as_float(whi[0]));
    o[2] = make_float4(__uint_as_float(whi[1]), __uint_as_float(whi[2]), __int_as_float(outref[0]),
                       __int_as_float(outref[1]));
    o[3] = make_float4(__int_as_float(outref[2]), __int_as_float(outref[3]), s[1], s[2]);
}

}  // namespace

size_t bvh4_scratch_bytes(int n) {
    const size_t ni = (size_t)(n > 1 ? n - 1 : 1);
    return 2 * ni * sizeof(int2) + 256;
}

size_t bvh4_node_capacity(int n) { return (size_t)(n > 1 ? n - 1 : 1) + 8; }

cudaError_t bvh4_build(const float4 *nodes2, int n, float4 *nodes4, void *scratch, uint32_t *status, int *count_out,
                       cudaStream_t s) {
    *count_out = 0;
    if (n <= 0) return cudaSuccess;
    const int ni = n > 1 ? n - 1 : 1;
    int2 *qa = (int2 *)scratch, *qb = qa + ni;
    unsigned *counters = (unsigned *)(qb + ni);  // [0] next-wave items, [1] nodes allocated
    const int2 root = make_int2(0, 0);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(qa, &root, sizeof(int2), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
    // node 0 is the root; node 1 pads the root's line, so the first allocation starts at 2
    const unsigned first = 2;
    if ((e = cudaMemcpyAsync(counters + 1, &first, sizeof(unsigned), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
    const int cap = (int)bvh4_node_capacity(n);
    int nin = 1, waves = 0;
    while (nin > 0) {
        if (++waves > 4 * 64 + 8) return cudaErrorInvalidValue;  // deeper than any LBVH of 2^32 leaves
        if ((e = cudaMemsetAsync(counters, 0, sizeof(unsigned), s)) != cudaSuccess) return e;
        k_collapse<<<(nin + kThreads4 - 1) / kThreads4, kThreads4, 0, s>>>(ni, nodes2, qa, nin, qb, counters,
                                                                           counters + 1, cap, ni, nodes4, status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        unsigned next = 0;
        if ((e = cudaMemcpyAsync(&next, counters, sizeof(unsigned), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        nin = (int)std::min<unsigned>(next, (unsigned)ni);
        int2 *t = qa;
        qa = qb;
        qb = t;
    }
    unsigned total = 0;
    if ((e = cudaMemcpyAsync(&total, counters + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    *count_out = (int)std::min<unsigned>(total, (unsigned)cap);
    return cudaSuccess;
}

}  // namespace hrt
