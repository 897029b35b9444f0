// hrt_ps_w4.cu -- launchers of the occupancy-oriented persistent 4-wide trace
// (k_diffuse_w4, hrt_trace_w4.cuh): accumulate, recording and statistics modes, for the
// resident-block / shared-stack shapes the tuner chooses from.  Kept in their own
// translation unit so that the build compiles them in parallel with the rest.
#include "hrt_trace_w4.cuh"

namespace hrt {

namespace {

// Blocks of a launch: one resident wave; with a lane budget, enough blocks that every ray
// id is taken even if each lane takes exactly its budget.
unsigned w4_grid(const DiffuseParams &p, int resident, int block) {
    if (!p.lane_budget) return (unsigned)resident;
    const unsigned long long nf = ((p.faces & 1) ? 1 : 0) + ((p.faces & 2) ? 1 : 0);
    const unsigned long long total = (unsigned long long)p.count * (unsigned long long)(p.dimx * p.dimy) * nf;
    const unsigned long long per_block = (unsigned long long)block * p.lane_budget;
    unsigned long long g = (total + per_block - 1) / per_block;
    if (g < (unsigned long long)resident) g = (unsigned long long)resident;
    if (g > 0x7FFFFFFFull) g = 0x7FFFFFFFull;
    return (unsigned)g;
}

template <int NB, bool RECORD, bool STATS, int MINB, int SD, int BLOCK, int KB = 1, bool MULTI = false, bool LIN = false>
cudaError_t w4_launch(const DiffuseParams &p, cudaStream_t s) {
    // resident blocks of one wave (SMs x blocks per SM); initialised once per instantiation,
    // thread-safe (the server launches from several threads)
    static const int resident = [] {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm,
                                                      k_diffuse_w4<NB, RECORD, STATS, MINB, SD, BLOCK, KB, MULTI, LIN>,
                                                      BLOCK, 0);
        return (sms < 1 ? 1 : sms) * (per_sm < 1 ? 1 : per_sm);
    }();
    cudaError_t e = cudaMemsetAsync(p.fetch, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    DiffuseParams q = p;
    q.refill = refill_threshold(false, true);
    k_diffuse_w4<NB, RECORD, STATS, MINB, SD, BLOCK, KB, MULTI, LIN><<<w4_grid(q, resident, BLOCK), BLOCK, 0, s>>>(q);
    return cudaGetLastError();
}

// The tuner's shapes: threads per block x resident blocks per SM (all 64 registers a thread
// but lean5, 48), shared stack entries per lane (a ring over local memory, or with LIN the
// bottom entries) and the warp's ray-id batch.
template <int NB, bool RECORD, bool STATS>
cudaError_t w4_shape(const DiffuseParams &p, int variant, cudaStream_t s) {
    switch (variant) {
        case DV_W4S5: return w4_launch<NB, RECORD, STATS, 5, 8, 256>(p, s);
        case DV_W4S4D16: return w4_launch<NB, RECORD, STATS, 4, 16, 256, 1, false, true>(p, s);
        case DV_W4S4D32: return w4_launch<NB, RECORD, STATS, 4, 32, 256, 1, false, true>(p, s);
        case DV_W4B128: return w4_launch<NB, RECORD, STATS, 8, 8, 128>(p, s);
        case DV_W4B512: return w4_launch<NB, RECORD, STATS, 2, 8, 512>(p, s);
        case DV_W4K4: return w4_launch<NB, RECORD, STATS, 4, 8, 256, 4>(p, s);
        case DV_W4K16: return w4_launch<NB, RECORD, STATS, 4, 8, 256, 16>(p, s);
        default: return w4_launch<NB, RECORD, STATS, 4, 8, 256>(p, s);
    }
}

}  // namespace

bool is_w4s_variant(int v) { return v >= DV_W4S4 && v <= DV_W4S4D32; }

cudaError_t launch_w4s(const DiffuseParams &p, int variant, cudaStream_t s) {
    if (!p.sc.nodes4 || p.sc.voxels) return cudaErrorInvalidValue;
    if (p.Bc <= 1) return w4_shape<1, false, false>(p, variant, s);
    if (p.Bc <= 2) return w4_shape<2, false, false>(p, variant, s);
    if (p.Bc <= 4) return w4_shape<4, false, false>(p, variant, s);
    if (p.Bc <= 8) return w4_shape<8, false, false>(p, variant, s);
    if (p.Bc <= 16) return w4_shape<16, false, false>(p, variant, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_w4s_record(const DiffuseParams &p, uint32_t *hits, int variant, cudaStream_t s) {
    if (!p.sc.nodes4 || p.sc.voxels) return cudaErrorInvalidValue;
    DiffuseParams q = p;
    q.hits = hits;
    q.Bc = 1;
    return w4_shape<1, true, false>(q, variant, s);
}

cudaError_t launch_w4s_multi_record(const DiffuseParams &p, cudaStream_t s) {
    if (!p.slots || p.nslots < 1 || p.nslots > kMaxSlots || p.lane_budget) return cudaErrorInvalidValue;
    if (p.multi_total == 0) return cudaSuccess;
    DiffuseParams q = p;
    q.Bc = 1;
    return w4_launch<1, true, false, 4, 8, 256, 1, true>(q, s);
}

cudaError_t launch_w4s_stats(const DiffuseParams &p, int variant, cudaStream_t s) {
    if (!p.sc.nodes4 || p.sc.voxels) return cudaErrorInvalidValue;
    if (p.Bc <= 1) return w4_shape<1, false, true>(p, variant, s);
    if (p.Bc <= 4) return w4_shape<4, false, true>(p, variant, s);
    return cudaErrorInvalidValue;
}

}  // namespace hrt
