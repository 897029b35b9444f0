// hrt_ps_special.cu -- persistent diffuse trace: scenes with voxels, traversal statistics
// and the recording mode of the batched sweep.
//
// Instantiations of k_diffuse_ps (hrt_trace.cuh), in their own translation unit so that
// the build compiles them in parallel with the rest.
#include "hrt_trace.cuh"

namespace hrt {

namespace {

template <int NB, bool RECORD, int MINB, bool VOX, bool W4, bool STATS>
cudaError_t ps_launch(const DiffuseParams &p, cudaStream_t s) {
    // resident blocks of one wave (SMs x blocks per SM); initialised once per instantiation,
    // thread-safe (the server launches from several threads)
    static const int resident = [] {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_diffuse_ps<NB, RECORD, MINB, VOX, W4, STATS>, kBlock, 0);
        return (sms < 1 ? 1 : sms) * (per_sm < 1 ? 1 : per_sm);
    }();
    cudaError_t e = cudaMemsetAsync(p.fetch, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    DiffuseParams q = p;
    q.refill = refill_threshold(VOX);
    k_diffuse_ps<NB, RECORD, MINB, VOX, W4, STATS><<<ps_grid(q, resident), kBlock, 0, s>>>(q);
    return cudaGetLastError();
}

template <int NB>
cudaError_t vox_variant(const DiffuseParams &p, int variant, cudaStream_t s) {
    if (variant == DV_W4 || variant == DV_W43) return ps_launch<NB, false, 4, true, true, false>(p, s);
    return ps_launch<NB, false, 4, true, false, false>(p, s);
}

}  // namespace

// Scenes with voxels: binary or 4-wide traversal, 4 resident blocks per SM.
cudaError_t launch_ps_voxels(const DiffuseParams &p, int variant, cudaStream_t s) {
    if (p.Bc <= 1) return vox_variant<1>(p, variant, s);
    if (p.Bc <= 2) return vox_variant<2>(p, variant, s);
    if (p.Bc <= 4) return vox_variant<4>(p, variant, s);
    if (p.Bc <= 8) return vox_variant<8>(p, variant, s);
    if (p.Bc <= 16) return vox_variant<16>(p, variant, s);
    return cudaErrorInvalidValue;
}

// Node-visit and primitive-test counting (into sc.visits) of the default 4-wide traversal,
// for up to 4 bands in flight.
cudaError_t launch_ps_stats(const DiffuseParams &p, cudaStream_t s) {
    if (p.sc.voxels) {
        if (p.Bc <= 1) return ps_launch<1, false, 4, true, true, true>(p, s);
        if (p.Bc <= 4) return ps_launch<4, false, 4, true, true, true>(p, s);
    } else {
        if (p.Bc <= 1) return ps_launch<1, false, 4, false, true, true>(p, s);
        if (p.Bc <= 4) return ps_launch<4, false, 4, false, true, true>(p, s);
    }
    return cudaErrorInvalidValue;
}

// Recording mode (one hit code per ray id, no sums) for the batched sweep.
cudaError_t launch_diffuse_record(const DiffuseParams &p, uint32_t *hits, int variant, cudaStream_t s) {
    if ((long long)p.count * p.dimx * p.dimy <= 0) return cudaSuccess;
    if (is_w4s_variant(variant) && p.sc.nodes4 && !p.sc.voxels) return launch_w4s_record(p, hits, variant, s);
    DiffuseParams q = p;
    q.hits = hits;
    q.Bc = 1;
    if ((variant == DV_W4 || variant == DV_W43 || is_w4s_variant(variant)) && !q.sc.nodes4) variant = DV_PS3;
    switch (variant) {
        case DV_W4: return ps_launch<1, true, 4, false, true, false>(q, s);
        case DV_W43: return ps_launch<1, true, 3, false, true, false>(q, s);
        case DV_PS4: return ps_launch<1, true, 4, false, false, false>(q, s);
        default: return ps_launch<1, true, 3, false, false, false>(q, s);
    }
}

}  // namespace hrt
