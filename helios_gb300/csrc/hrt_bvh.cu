// hrt_bvh.cu -- LBVH build over patches, triangles, disks and voxels.
//
// Replaces the reference's acceleration-structure build (OptiX GAS over AABB
// custom primitives, plugins/radiation/src/backends/OptiX8Backend.cpp:1382-1507).
// Stages, all on one stream:
//   1. k_records   : intersection + ray-origin records and AABBs from the 4x4 transforms
//   2. k_bounds_*  : centroid and scene bounds (exact min/max reduction)
//   3. k_morton    : 63-bit Morton codes (21 bits per axis) of the AABB centroids, bit 63
//                    set for voxels (they form their own subtree)
//   4. radix sort  : stable LSD, 8 passes of 8 bits over (code, index) pairs
//   5. k_karras    : binary radix tree (Karras, HPG 2012), ties broken by index
//   6. k_leaves    : padded leaf boxes and records in leaf order
//   7. k_refit     : bottom-up box refit (atomic arrival counters), packed nodes
// Every stage is integer work or exact min/max except the per-primitive record
// arithmetic, which follows the fixed FP32 sequences of hrt_device.cuh, so the
// result is bit-identical to a host build of the same algorithm.
#include <cstdlib>

#include "hrt_device.cuh"
#include "hrt_internal.h"

namespace hrt {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = kSortTile / kThreads;  // 8

__global__ void k_records(int n, const float *__restrict__ T, const uint32_t *__restrict__ type,
                          const float *__restrict__ lad, float4 *__restrict__ rec_tmp, float4 *__restrict__ rgen,
                          float *__restrict__ aabb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float t[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) t[k] = T[16 * (size_t)i + k];
    float4 rec[4], g[4];
    f3 lo, hi;
    make_records(t, type[i], lad ? lad[i] : 0.f, rec, g, &lo, &hi);
    rec[1].w = __uint_as_float((uint32_t)i);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        rec_tmp[4 * (size_t)i + k] = rec[k];
        rgen[4 * (size_t)i + k] = g[k];
    }
    float *a = aabb + 6 * (size_t)i;
    a[0] = lo.x;
    a[1] = lo.y;
    a[2] = lo.z;
    a[3] = hi.x;
    a[4] = hi.y;
    a[5] = hi.z;
}

// Per-block partial bounds: [clo3, chi3, blo3, bhi3].
__global__ void k_bounds_partial(int n, const float *__restrict__ aabb, float *__restrict__ partial) {
    float v[12];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        v[k] = INFINITY;
        v[3 + k] = -INFINITY;
        v[6 + k] = INFINITY;
        v[9 + k] = -INFINITY;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float *a = aabb + 6 * (size_t)i;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float c = (a[k] + a[3 + k]) * 0.5f;
            v[k] = fminf(v[k], c);
            v[3 + k] = fmaxf(v[3 + k], c);
            v[6 + k] = fminf(v[6 + k], a[k]);
            v[9 + k] = fmaxf(v[9 + k], a[3 + k]);
        }
    }
    __shared__ float sh[12][kThreads];
#pragma unroll
    for (int k = 0; k < 12; ++k) sh[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                float a = sh[k][threadIdx.x], b = sh[k][threadIdx.x + s];
                bool mx = (k >= 3 && k < 6) || k >= 9;
                sh[k][threadIdx.x] = mx ? fmaxf(a, b) : fminf(a, b);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 12) partial[12 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

// Final bounds: out[0..2] clo, [3..5] chi, [6..8] blo, [9..11] bhi, [12..14] Morton scale, [15] extent.
__global__ void k_bounds_final(int nparts, const float *__restrict__ partial, float *__restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float v[12];
    for (int k = 0; k < 12; ++k) v[k] = partial[k];
    for (int p = 1; p < nparts; ++p)
        for (int k = 0; k < 12; ++k) {
            float b = partial[12 * p + k];
            bool mx = (k >= 3 && k < 6) || k >= 9;
            v[k] = mx ? fmaxf(v[k], b) : fminf(v[k], b);
        }
    float ext = 0.f;
    for (int k = 0; k < 3; ++k) {
        out[k] = v[k];
        out[3 + k] = v[3 + k];
        out[6 + k] = v[6 + k];
        out[9 + k] = v[9 + k];
        ext = fmaxf(ext, v[9 + k] - v[6 + k]);
        float e = v[3 + k] - v[k];
        out[12 + k] = (e > 0.f) ? (2097152.0f / e) : 0.f;
    }
    out[15] = ext;
}

__device__ __forceinline__ uint64_t expand21(uint32_t v) {
    uint64_t x = v & 0x1FFFFFu;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}
__device__ __forceinline__ uint32_t quant21(float c, float lo, float scale) {
    float q = (c - lo) * scale;
    if (!(q > 0.f)) q = 0.f;
    if (q > 2097151.0f) q = 2097151.0f;
    return (uint32_t)q;
}

// Bit 63 (above the 63 Morton bits) marks voxels: sorted after the surfaces, they form the
// root's second subtree, so their large boxes do not widen the nodes over the leaves.
__global__ void k_morton(int n, const float *__restrict__ aabb, const float *__restrict__ bnd,
                         const uint32_t *__restrict__ type, uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *a = aabb + 6 * (size_t)i;
    uint64_t code = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float c = (a[k] + a[3 + k]) * 0.5f;
        code |= expand21(quant21(c, bnd[k], bnd[12 + k])) << (2 - k);
    }
    if (type[i] == PT_VOXEL) code |= 1ull << 63;
    keys[i] = code;
    vals[i] = (uint32_t)i;
}

// ---------------------------------------------------------------- radix sort
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total, uint32_t *sh_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) sh_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = (lane < (int)(blockDim.x >> 5)) ? sh_warp[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += y;
        }
        sh_warp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    uint32_t before = (warp > 0 ? sh_warp[warp - 1] : 0u) + x - v;
    *total = sh_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

__global__ void k_hist(int n, const uint64_t *__restrict__ keys, int shift, int nblk, uint32_t *__restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int base = blockIdx.x * kSortTile;
    for (int k = threadIdx.x; k < kSortTile; k += kThreads) {
        int i = base + k;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_scan_blocks(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, int count,
                              uint32_t *__restrict__ sums) {
    __shared__ uint32_t shw[32];
    int base = blockIdx.x * kSortTile;
    uint32_t v[kItems];
    uint32_t loc = 0;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        int i = base + threadIdx.x * kItems + j;
        v[j] = (i < count) ? in[i] : 0u;
        loc += v[j];
    }
    uint32_t tot;
    uint32_t run = block_excl_scan(loc, &tot, shw);
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        int i = base + threadIdx.x * kItems + j;
        if (i < count) out[i] = run;
        run += v[j];
    }
    if (threadIdx.x == 0 && sums) sums[blockIdx.x] = tot;
}

__global__ void k_scan_add(uint32_t *__restrict__ out, int count, const uint32_t *__restrict__ sums) {
    int base = blockIdx.x * kSortTile;
    uint32_t add = sums[blockIdx.x];
    for (int k = threadIdx.x; k < kSortTile; k += kThreads) {
        int i = base + k;
        if (i < count) out[i] += add;
    }
}

__global__ void k_scatter(int n, const uint64_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                          uint64_t *__restrict__ kout, uint32_t *__restrict__ vout, int shift, int nblk,
                          const uint32_t *__restrict__ offs) {
    __shared__ uint64_t sk[kSortTile];
    __shared__ uint32_t sv[kSortTile];
    __shared__ uint32_t shw[32];
    __shared__ uint32_t dstart[256];
    __shared__ uint32_t dcount[256];
    const int base = blockIdx.x * kSortTile;
    uint64_t k[kItems];
    uint32_t v[kItems];
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        int i = base + threadIdx.x * kItems + j;
        k[j] = (i < n) ? kin[i] : ~0ull;
        v[j] = (i < n) ? vin[i] : 0u;
    }
    // 8 stable 1-bit splits sort the tile by the current digit.
    for (int b = 0; b < 8; ++b) {
        int bit = shift + b;
        uint32_t z = 0;
#pragma unroll
        for (int j = 0; j < kItems; ++j) z += ((k[j] >> bit) & 1ull) ? 0u : 1u;
        uint32_t ztot;
        uint32_t zb = block_excl_scan(z, &ztot, shw);
        uint32_t zr = zb;
#pragma unroll
        for (int j = 0; j < kItems; ++j) {
            uint32_t idx = threadIdx.x * kItems + j;
            bool one = (k[j] >> bit) & 1ull;
            uint32_t pos = one ? (ztot + (idx - zr)) : zr;
            if (!one) ++zr;
            sk[pos] = k[j];
            sv[pos] = v[j];
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kItems; ++j) {
            k[j] = sk[threadIdx.x * kItems + j];
            v[j] = sv[threadIdx.x * kItems + j];
        }
        __syncthreads();
    }
    dcount[threadIdx.x] = 0;
    __syncthreads();
    const int valid = min(kSortTile, n - base);
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        int idx = threadIdx.x * kItems + j;
        if (idx < valid) atomicAdd(&dcount[(k[j] >> shift) & 255u], 1u);
    }
    __syncthreads();
    uint32_t tot;
    uint32_t st = block_excl_scan(dcount[threadIdx.x], &tot, shw);
    dstart[threadIdx.x] = st;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        int idx = threadIdx.x * kItems + j;
        if (idx < valid) {
            uint32_t d = (k[j] >> shift) & 255u;
            uint32_t pos = offs[d * nblk + blockIdx.x] + (idx - dstart[d]);
            kout[pos] = k[j];
            vout[pos] = v[j];
        }
    }
}

// Exclusive scan of `count` u32 values (count <= kSortTile^2).
cudaError_t scan_u32(const uint32_t *in, uint32_t *out, int count, uint32_t *tmp, cudaStream_t s) {
    int nb = (count + kSortTile - 1) / kSortTile;
    if (nb <= 1) {
        k_scan_blocks<<<1, kThreads, 0, s>>>(in, out, count, nullptr);
        return cudaGetLastError();
    }
    uint32_t *sums = tmp, *sums_scan = tmp + nb;
    k_scan_blocks<<<nb, kThreads, 0, s>>>(in, out, count, sums);
    k_scan_blocks<<<1, kThreads, 0, s>>>(sums, sums_scan, nb, nullptr);
    k_scan_add<<<nb, kThreads, 0, s>>>(out, count, sums_scan);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- hierarchy
__device__ __forceinline__ int delta(const uint64_t *__restrict__ c, int n, int i, int j) {
    if (j < 0 || j > n - 1) return -1;
    uint64_t a = c[i], b = c[j];
    if (a == b) return 64 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clzll(a ^ b);
}

__global__ void k_karras(int n, const uint64_t *__restrict__ codes, int32_t *__restrict__ child,
                         int32_t *__restrict__ parent_int, int32_t *__restrict__ parent_leaf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int dsgn = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(codes, n, i, i - dsgn);
    int lmax = 2;
    while (delta(codes, n, i, i + lmax * dsgn) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(codes, n, i, i + (l + t) * dsgn) > dmin) l += t;
    int j = i + l * dsgn;
    int dnode = delta(codes, n, i, j);
    int sp = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(codes, n, i, i + (sp + t) * dsgn) > dnode) sp += t;
    } while (t > 1);
    int gamma = i + sp * dsgn + min(dsgn, 0);
    int lo = min(i, j), hi = max(i, j);
    if (lo == gamma) {
        child[2 * i] = ~gamma;
        parent_leaf[gamma] = i;
    } else {
        child[2 * i] = gamma;
        parent_int[gamma] = i;
    }
    if (hi == gamma + 1) {
        child[2 * i + 1] = ~(gamma + 1);
        parent_leaf[gamma + 1] = i;
    } else {
        child[2 * i + 1] = gamma + 1;
        parent_int[gamma + 1] = i;
    }
    if (i == 0) parent_int[0] = -1;
}

__global__ void k_leaves(int n, const uint32_t *__restrict__ perm, const float4 *__restrict__ rec_tmp,
                         const float *__restrict__ aabb, const float *__restrict__ bnd, float4 *__restrict__ rec,
                         float *__restrict__ leafbox) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t p = perm[i];
    float ext = bnd[15];
#pragma unroll
    for (int k = 0; k < 4; ++k) rec[4 * (size_t)i + k] = rec_tmp[4 * (size_t)p + k];
    const float *a = aabb + 6 * (size_t)p;
    float *o = leafbox + 6 * (size_t)i;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        o[k] = pad_lo(a[k], ext);
        o[3 + k] = pad_hi(a[3 + k], ext);
    }
}

__device__ __forceinline__ void load_box(int32_t c, const float *leafbox, const float *nodebox, float *b) {
    const float *src = (c < 0) ? (leafbox + 6 * (size_t)(~c)) : (nodebox + 6 * (size_t)c);
#pragma unroll
    for (int k = 0; k < 6; ++k) b[k] = __ldcg(src + k);
}

__device__ __forceinline__ void write_node(float4 *nodes, int idx, const float *b0, const float *b1, int32_t c0,
                                           int32_t c1) {
    float4 *o = nodes + 4 * (size_t)idx;
    o[0] = make_float4(b0[0], b0[1], b0[2], b0[3]);
    o[1] = make_float4(b0[4], b0[5], b1[0], b1[1]);
    o[2] = make_float4(b1[2], b1[3], b1[4], b1[5]);
    o[3] = make_float4(__int_as_float(c0), __int_as_float(c1), 0.f, 0.f);
}

__global__ void k_refit(int n, const int32_t *__restrict__ parent_leaf, const int32_t *__restrict__ parent_int,
                        const int32_t *__restrict__ child, const float *__restrict__ leafbox, float *nodebox,
                        uint32_t *flags, float4 *__restrict__ nodes, uint32_t *status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = parent_leaf[i];
    for (int steps = 0; node >= 0; ++steps) {
        if (node >= n - 1 || steps > 256) {  // a Karras tree over <= 2^32 keys is at most 96 deep
            atomicOr(status, 8u);
            return;
        }
        __threadfence();
        uint32_t arrived = atomicAdd(&flags[node], 1u);
        if (arrived == 0) return;  // the sibling subtree finishes this node
        __threadfence();
        int32_t c0 = child[2 * node], c1 = child[2 * node + 1];
        float b0[6], b1[6], u[6];
        load_box(c0, leafbox, nodebox, b0);
        load_box(c1, leafbox, nodebox, b1);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            u[k] = fminf(b0[k], b1[k]);
            u[3 + k] = fmaxf(b0[3 + k], b1[3 + k]);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) __stcg(nodebox + 6 * (size_t)node + k, u[k]);
        write_node(nodes, node, b0, b1, c0, c1);
        node = parent_int[node];
    }
}

__global__ void k_single(const float *__restrict__ leafbox, float4 *__restrict__ nodes) {
    float b1[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    float b0[6];
    for (int k = 0; k < 6; ++k) b0[k] = leafbox[k];
    write_node(nodes, 0, b0, b1, ~0, kEmptyChild);
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// ---------------------------------------------------------------- PLOC
// Agglomerative clustering of the Morton-ordered leaves (Meister & Bittner, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction", TVCG 2018): each
// cluster finds the neighbour within +-kPlocRadius places whose merged box has the least
// surface area (ties: the smaller index); mutual pairs merge into a new binary node; the
// survivors are compacted in order; repeat until one cluster is left.  Node indices are
// handed out from n-2 downwards by a prefix sum, so the root is node 0 and the tree does not
// depend on scheduling.  The leaves are the same record slots as the LBVH's.  Search radius
// 64; measured on the 1 M-triangle orchard (node visits per ray, G rays/s): 16 40.6 / 1.64,
// 32 39.4 / 1.93, 64 38.9 / 1.98, 128 38.2 / 1.97.  HRT_PLOC_RADIUS overrides (1-256).
constexpr int kPlocRadius = 64;

__device__ __forceinline__ float merged_area(const float *a, const float *b) {
    const float dx = fmaxf(a[3], b[3]) - fminf(a[0], b[0]);
    const float dy = fmaxf(a[4], b[4]) - fminf(a[1], b[1]);
    const float dz = fmaxf(a[5], b[5]) - fminf(a[2], b[2]);
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_ploc_init(int n, const float *__restrict__ leafbox, float *__restrict__ cbox,
                            int32_t *__restrict__ cid) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
#pragma unroll
    for (int k = 0; k < 6; ++k) cbox[6 * (size_t)i + k] = leafbox[6 * (size_t)i + k];
    cid[i] = ~i;
}

__global__ void k_ploc_nn(int m, int radius, const float *__restrict__ cbox, int32_t *__restrict__ nn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    float a[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) a[k] = cbox[6 * (size_t)i + k];
    float best = INFINITY;
    int bj = -1;
    const int lo = i - radius < 0 ? 0 : i - radius;
    const int hi = i + radius > m - 1 ? m - 1 : i + radius;
    for (int j = lo; j <= hi; ++j) {
        if (j == i) continue;
        float b[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) b[k] = __ldg(cbox + 6 * (size_t)j + k);
        const float d = merged_area(a, b);
        if (d < best) {  // j ascends: equal areas keep the smaller index
            best = d;
            bj = j;
        }
    }
    nn[i] = bj;
}

// create[i] = 1 when cluster i starts a mutual pair (i < nn[i]); keep[i] = 0 for the partner.
__global__ void k_ploc_flags(int m, const int32_t *__restrict__ nn, uint32_t *__restrict__ create,
                             uint32_t *__restrict__ keep) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int j = nn[i];
    const bool mutual = j >= 0 && j < m && nn[j] == i;
    create[i] = (mutual && i < j) ? 1u : 0u;
    keep[i] = (mutual && i > j) ? 0u : 1u;
}

__global__ void k_ploc_merge(int m, const int32_t *__restrict__ nn, const uint32_t *__restrict__ create,
                             const uint32_t *__restrict__ rank, int next_free, float *__restrict__ cbox,
                             int32_t *__restrict__ cid, float4 *__restrict__ nodes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || !create[i]) return;
    const int j = nn[i];
    const int node = next_free - (int)rank[i];
    float a[6], b[6], u[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        a[k] = cbox[6 * (size_t)i + k];
        b[k] = cbox[6 * (size_t)j + k];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        u[k] = fminf(a[k], b[k]);
        u[3 + k] = fmaxf(a[3 + k], b[3 + k]);
    }
    write_node(nodes, node, a, b, cid[i], cid[j]);
#pragma unroll
    for (int k = 0; k < 6; ++k) cbox[6 * (size_t)i + k] = u[k];
    cid[i] = node;
}

__global__ void k_ploc_compact(int m, const uint32_t *__restrict__ keep, const uint32_t *__restrict__ pos,
                               const float *__restrict__ cbox, const int32_t *__restrict__ cid,
                               float *__restrict__ cbox2, int32_t *__restrict__ cid2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || !keep[i]) return;
    const uint32_t o = pos[i];
#pragma unroll
    for (int k = 0; k < 6; ++k) cbox2[6 * (size_t)o + k] = cbox[6 * (size_t)i + k];
    cid2[o] = cid[i];
}

}  // namespace

size_t bvh_scratch_bytes(int n) { return bvh_scratch_bytes_c(n); }

void bvh_carve(BvhBuffers &bb, void *scratch, int n) {
    size_t nn = (size_t)(n > 1 ? n : 1);
    size_t ni = (size_t)(n > 1 ? n - 1 : 1);
    size_t nblk = (nn + kSortTile - 1) / kSortTile;
    size_t nh = 256 * nblk;
    char *p = (char *)scratch;
    auto take = [&](size_t bytes) {
        char *r = p;
        p += align256(bytes);
        return (void *)r;
    };
    bb.rec_tmp = (float4 *)take(nn * 4 * sizeof(float4));
    bb.aabb = (float *)take(nn * 6 * sizeof(float));
    bb.leafbox = (float *)take(nn * 6 * sizeof(float));
    bb.nodebox = (float *)take(ni * 6 * sizeof(float));
    bb.bounds = (float *)take(16 * sizeof(float));
    bb.partial = (float *)take(1024 * 12 * sizeof(float));
    bb.keys_alt = (uint64_t *)take(nn * sizeof(uint64_t));
    bb.vals_alt = (uint32_t *)take(nn * sizeof(uint32_t));
    bb.hist = (uint32_t *)take(nh * sizeof(uint32_t));
    bb.offs = (uint32_t *)take(nh * sizeof(uint32_t));
    bb.scan_tmp = (uint32_t *)take((2 * ((nh + kSortTile - 1) / kSortTile) + 64) * sizeof(uint32_t));
    bb.child = (int32_t *)take(2 * ni * sizeof(int32_t));
    bb.parent_int = (int32_t *)take(ni * sizeof(int32_t));
    bb.parent_leaf = (int32_t *)take(nn * sizeof(int32_t));
    bb.flags = (uint32_t *)take(ni * sizeof(uint32_t));
}

cudaError_t bvh_build(const float *T, const uint32_t *type, const float *lad, int n, BvhBuffers &b, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (n > 33000000) return cudaErrorInvalidValue;  // radix-sort offset scan covers 2048^2 bins
    const int grid = (n + kThreads - 1) / kThreads;
    k_records<<<grid, kThreads, 0, s>>>(n, T, type, lad, b.rec_tmp, b.rgen, b.aabb);
    int nparts = grid < 1024 ? grid : 1024;
    k_bounds_partial<<<nparts, kThreads, 0, s>>>(n, b.aabb, b.partial);
    k_bounds_final<<<1, 32, 0, s>>>(nparts, b.partial, b.bounds);
    k_morton<<<grid, kThreads, 0, s>>>(n, b.aabb, b.bounds, type, b.codes, b.perm);
    // 8 LSD passes; even pass count leaves the result in (codes, perm).
    const int nblk = (n + kSortTile - 1) / kSortTile;
    const int nh = 256 * nblk;
    uint32_t *offs = b.offs;
    uint64_t *ka = b.codes, *kb = b.keys_alt;
    uint32_t *va = b.perm, *vb = b.vals_alt;
    for (int pass = 0; pass < 8; ++pass) {
        int shift = 8 * pass;
        k_hist<<<nblk, kThreads, 0, s>>>(n, ka, shift, nblk, b.hist);
        cudaError_t e = scan_u32(b.hist, offs, nh, b.scan_tmp, s);
        if (e != cudaSuccess) return e;
        k_scatter<<<nblk, kThreads, 0, s>>>(n, ka, va, kb, vb, shift, nblk, offs);
        uint64_t *tk = ka;
        ka = kb;
        kb = tk;
        uint32_t *tv = va;
        va = vb;
        vb = tv;
    }
    k_leaves<<<grid, kThreads, 0, s>>>(n, b.perm, b.rec_tmp, b.aabb, b.bounds, b.rec, b.leafbox);
    if (n == 1) {
        k_single<<<1, 1, 0, s>>>(b.leafbox, b.nodes);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(b.flags, 0, sizeof(uint32_t) * (size_t)(n - 1), s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(b.parent_leaf, 0xFF, sizeof(int32_t) * (size_t)n, s);  // -1 = no parent yet
    if (e != cudaSuccess) return e;
    int gi = (n - 1 + kThreads - 1) / kThreads;
    k_karras<<<gi, kThreads, 0, s>>>(n, b.codes, b.child, b.parent_int, b.parent_leaf);
    k_refit<<<grid, kThreads, 0, s>>>(n, b.parent_leaf, b.parent_int, b.child, b.leafbox, b.nodebox, b.flags,
                                      b.nodes, b.status);
    return cudaGetLastError();
}

// Exclusive scan of any length (tiles of kSortTile, sums scanned recursively); tmp holds
// ploc_scan_tmp(count) words.
static size_t scan_tmp_words(int count) {
    size_t w = 64;
    for (int c = count; c > kSortTile;) {
        const int nb = (c + kSortTile - 1) / kSortTile;
        w += 2 * (size_t)nb;
        c = nb;
    }
    return w;
}

static cudaError_t scan_any(const uint32_t *in, uint32_t *out, int count, uint32_t *tmp, cudaStream_t s) {
    const int nb = (count + kSortTile - 1) / kSortTile;
    if (nb <= 1) {
        k_scan_blocks<<<1, kThreads, 0, s>>>(in, out, count, nullptr);
        return cudaGetLastError();
    }
    uint32_t *sums = tmp, *sums_scan = tmp + nb;
    k_scan_blocks<<<nb, kThreads, 0, s>>>(in, out, count, sums);
    cudaError_t e = scan_any(sums, sums_scan, nb, tmp + 2 * nb, s);
    if (e != cudaSuccess) return e;
    k_scan_add<<<nb, kThreads, 0, s>>>(out, count, sums_scan);
    return cudaGetLastError();
}

size_t ploc_scratch_bytes(int n) {
    const size_t nn = (size_t)(n > 1 ? n : 1);
    return 2 * align256(nn * 6 * sizeof(float)) + 2 * align256(nn * sizeof(int32_t)) +
           4 * align256(nn * sizeof(uint32_t)) + align256(scan_tmp_words(n) * sizeof(uint32_t));
}

static int ploc_radius() {
    static const int v = [] {  // initialised once, thread-safe
        const char *e = getenv("HRT_PLOC_RADIUS");
        const int r = e ? atoi(e) : kPlocRadius;
        return (r < 1 || r > 256) ? kPlocRadius : r;
    }();
    return v;
}

cudaError_t ploc_build(const float *leafbox, int n, float4 *nodes, void *scratch, cudaStream_t s) {
    if (n <= 1) return cudaSuccess;
    const int radius = ploc_radius();
    const size_t nn = (size_t)n;
    char *p = (char *)scratch;
    auto take = [&](size_t bytes) {
        char *r = p;
        p += align256(bytes);
        return (void *)r;
    };
    float *box[2] = {(float *)take(nn * 6 * sizeof(float)), (float *)take(nn * 6 * sizeof(float))};
    int32_t *cid[2] = {(int32_t *)take(nn * sizeof(int32_t)), (int32_t *)take(nn * sizeof(int32_t))};
    int32_t *nn_idx = (int32_t *)take(nn * sizeof(int32_t));
    uint32_t *create = (uint32_t *)take(nn * sizeof(uint32_t));
    uint32_t *rank = (uint32_t *)take(nn * sizeof(uint32_t));
    uint32_t *keep = (uint32_t *)take(nn * sizeof(uint32_t));
    uint32_t *tmp = (uint32_t *)take(scan_tmp_words(n) * sizeof(uint32_t));
    uint32_t *pos = create;  // reused after the merge
    k_ploc_init<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(n, leafbox, box[0], cid[0]);
    int m = n, cur = 0, next_free = n - 2;
    for (int iter = 0; m > 1; ++iter) {
        if (iter > 4 * 1024) return cudaErrorInvalidValue;  // each round merges at least one pair
        const int g = (m + kThreads - 1) / kThreads;
        k_ploc_nn<<<g, kThreads, 0, s>>>(m, radius, box[cur], nn_idx);
        k_ploc_flags<<<g, kThreads, 0, s>>>(m, nn_idx, create, keep);
        cudaError_t e = scan_any(create, rank, m, tmp, s);
        if (e != cudaSuccess) return e;
        uint32_t h[2];  // merges this round: last rank + last flag
        if ((e = cudaMemcpyAsync(&h[0], rank + (m - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return e;
        if ((e = cudaMemcpyAsync(&h[1], create + (m - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return e;
        k_ploc_merge<<<g, kThreads, 0, s>>>(m, nn_idx, create, rank, next_free, box[cur], cid[cur], nodes);
        if ((e = scan_any(keep, pos, m, tmp, s)) != cudaSuccess) return e;
        k_ploc_compact<<<g, kThreads, 0, s>>>(m, keep, pos, box[cur], cid[cur], box[1 - cur], cid[1 - cur]);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        const int merged = (int)(h[0] + h[1]);
        if (merged <= 0) return cudaErrorInvalidValue;
        next_free -= merged;
        m -= merged;
        cur = 1 - cur;
    }
    return next_free == -1 ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace hrt
