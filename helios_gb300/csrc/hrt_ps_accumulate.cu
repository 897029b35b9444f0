// hrt_ps_accumulate.cu -- persistent diffuse trace, accumulate mode, scenes without voxels.
//
// Instantiations of k_diffuse_ps (hrt_trace.cuh) for 1-16 bands in flight and the four
// traversal variants the tuner chooses from: binary or compressed 4-wide nodes, with 4 or 3
// resident blocks per SM.  Kept in their own translation unit so that the build compiles
// them in parallel with the rest.
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
cudaError_t by_variant(const DiffuseParams &p, int variant, cudaStream_t s) {
    switch (variant) {
        case DV_W4: return ps_launch<NB, false, 4, false, true, false>(p, s);
        case DV_W43: return ps_launch<NB, false, 3, false, true, false>(p, s);
        case DV_PS3: return ps_launch<NB, false, 3, false, false, false>(p, s);
        default: return ps_launch<NB, false, 4, false, false, false>(p, s);
    }
}

}  // namespace

cudaError_t launch_ps_accumulate(const DiffuseParams &p, int variant, cudaStream_t s) {
    if (p.Bc <= 1) return by_variant<1>(p, variant, s);
    if (p.Bc <= 2) return by_variant<2>(p, variant, s);
    if (p.Bc <= 4) return by_variant<4>(p, variant, s);
    if (p.Bc <= 8) return by_variant<8>(p, variant, s);
    if (p.Bc <= 16) return by_variant<16>(p, variant, s);
    return cudaErrorInvalidValue;
}

}  // namespace hrt
