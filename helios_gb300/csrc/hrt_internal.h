// hrt_internal.h -- structures shared by the CUDA translation units of libhrt.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "hrt_device.cuh"

namespace hrt {

// Scene as the trace kernels see it.
struct TraceScene {
    const float4 *rec;    // [n*4] intersection records, BVH leaf order
    const float4 *nodes;  // [max(n-1,1)*4] BVH2 nodes
    const float4 *nodes4; // [n4*4] compressed 4-wide nodes (hrt_device.cuh), root 0
    int n4;
    const float4 *rgen;   // [n*4] ray-origin records, original order
    const float4 *bbox;   // [nbbox*4] periodic wall corners (xyz, w unused)
    int n;
    int nbbox;
    int voxels;           // the scene holds voxel primitives
    float periodic_x, periodic_y;
    const int8_t *twosided; // [n] two-sided flags
    uint32_t *status;     // device error word (ERR_* bits)
    unsigned long long *rays; // traced-ray counter
    unsigned long long *visits; // [2] node visits, primitive tests (statistics launches only)
    MaskSet masks;        // texture masks (masks.id null: none)
    const uint32_t *cover; // [n] bit s: a translucent cover for this launch's rays of source s (null: none)
    uint32_t visit_budget; // node visits one ray segment may make before it is ended with ERR_BOUNDS
                           // (2n+64 by default: a ray visits each node at most once)
};

// Translucent covers of one launch: sheet optics and the cover deposits.
constexpr int kGlassBands = 16;  // launched bands a launch with covers can carry
struct GlassParams {
    const float *gn, *gkl;     // [gS*n*Bg] refractive index, absorption product K*L
    const uint8_t *flags;      // [Bg] band flags of this launch (device)
    int Bg, Bl;
    int sky;                   // diffuse: some launched band has sky flux (covers then take deposits)
    double *rin, *stop, *sbot; // [n*Bl] absorbed / reflected shares deposited on covers
    double *Gcov;              // direct: [n*S*2*Bl] strength x transmittance of unoccluded rays that crossed covers
    const float *src_flux;     // direct: [S*Bl]
};

// Radiation source in device form (rotation pre-expanded to a 3x3 matrix on the host).
struct SourceDev {
    int type;             // 0 collimated, 1 sphere, 2 sun sphere, 3 rectangle, 4 disk
    float pos[3];
    float w0, w1;
    float R[9];
};

// Ray ids inside one trace launch are 32-bit (primitive x stratum x face, and the
// persistent kernel's per-face id range).  A pass whose primitives x rays per primitive x
// faces reaches kLaunchRayLimit runs as consecutive launches over primitive chunks, so
// every launch's ids stay below 2^31 and no 32-bit product or grid-stride step wraps.
constexpr uint64_t kLaunchRayLimit = 1ull << 31;

// Primitives per launch for `rays_per_primitive` rays each under `limit` rays per launch;
// 0 when a single primitive's rays alone exceed the limit (or the limit is 0).
inline uint32_t launch_chunk_prims(uint64_t rays_per_primitive, uint64_t limit) {
    if (limit > kLaunchRayLimit) limit = kLaunchRayLimit;
    if (rays_per_primitive == 0) return 0xFFFFFFFFu;
    const uint64_t c = limit / rays_per_primitive;
    return c > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)c;
}

struct DirectParams {
    TraceScene sc;
    const SourceDev *src;
    int S;
    int dimx, dimy;
    uint32_t seed, pass;
    uint32_t offset, count;   // primitive range
    double *G;                // [n*S*2] sums of strength of unoccluded rays, [p][s][face]
    GlassParams gl;           // launches with covers (sc.cover non-null)
};

struct SkyParams {
    const float *flux;     // [Bc] diffuse flux per compacted band
    const float *K;        // [Bc] power-law exponent (0 = off)
    const float *knorm;    // [Bc]
    const float *peak;     // [Bc*3]
    const float *prague;   // [Bc*4]
};

// One scene of a multi-scene recording launch (k_diffuse_w4 MULTI): its trace scene, the
// primitive chunk and ray counts of its pass, and the launch's ray ids [id_begin, id_begin +
// count * dimx * dimy * faces) that belong to it.
struct SceneSlot {
    TraceScene sc;
    int dimx, dimy;
    uint32_t seed, pass;
    uint32_t offset, count;          // primitive chunk (count x rays x faces < 2^31)
    unsigned long long id_begin;
    uint32_t *hits;                  // [face][n][R] hit codes of this scene
};
constexpr int kMaxSlots = 32;        // scenes (chunks) one multi-scene launch carries

struct DiffuseParams {
    TraceScene sc;
    int dimx, dimy;
    uint32_t seed, pass;
    uint32_t offset, count;
    int faces;                // bit 0: launch top face (1), bit 1: launch bottom face (0)
    int Bc;                   // compacted (launched) band count
    int Bl;                   // buffer stride
    const float *otop, *obot; // radiation_out [n*Bl]
    SkyParams sky;
    double *Gt, *Gb;          // [n*Bl] sums of incoming values per origin face
    unsigned long long *fetch; // ray-id counter of the persistent kernel (zeroed by the launcher)
    uint32_t lane_budget;      // persistent kernel: rays a lane takes before its block retires
                               // (0 = no limit: one resident wave of blocks runs to the end)
    uint32_t *hits;            // record mode: hit code per ray id, else unused
    int refill = 0;            // persistent kernel: a warp leaves its node loop to give idle lanes new
                               // rays when fewer than this many lanes are still in it (0: never);
                               // set by the launcher
    GlassParams gl;            // launches with covers (sc.cover non-null)
    const SceneSlot *slots = nullptr;     // multi-scene recording: [nslots] device table
    int nslots = 0;
    unsigned long long multi_total = 0;   // ray ids of all slots
};

// ---------------------------------------------------------------- cameras
struct CameraParams {
    TraceScene sc;
    float pos[3];
    float M[9];                // camera-to-world rotation, row-major; column 0 is the view axis
    float focal, lens, inv_aspect, viewplane;
    int W, H;                  // full image
    int ox, oy, tw, th;        // this launch's tile: first pixel and size
    int aa;                    // rays per pixel
    uint32_t seed, cam_id;
    int Bl, S;
    const SourceDev *src;      // [S]
    const float *src_flux;     // [S*Bl]
    const float *otop, *obot;  // radiation_out [n*Bl]
    SkyParams sky;             // camera sky: peak = sun direction per band, Prague parameters
    const float *sky_rad, *disk_rad, *dflux;  // [Bl] each, or null
    const uint32_t *emission;  // [Bl] or null
    float sun[3], disk_cos;
    double *pix;               // [W*H*Bl] accumulated radiance
    uint32_t *labels;          // [W*H]
    float *depths;             // [W*H]
};
cudaError_t launch_camera(const CameraParams &p, int max_blocks, cudaStream_t s);
cudaError_t launch_pixel_labels(const CameraParams &p, cudaStream_t s);
cudaError_t launch_add(double *dst, const double *src, size_t n, cudaStream_t s);
// Camera-to-world rotation for a view axis of the given zenith and azimuth (host, FP64 rounded to FP32).
void camera_rotation(float zenith, float azimuth, float M[9]);

// ---------------------------------------------------------------- energy balance
struct EnergyParams {
    int n;
    const float *R;            // [n] absorbed radiation, sum over bands
    const float *Tin;          // [n] previous / initial surface temperature
    const float *Ta, *ea, *press, *gH, *gS, *eps, *Qother, *cap, *hs, *sided;  // [n] each
    const uint8_t *nsides;     // [n] 1 or 2
    float dt;                  // > 0: storage term over this time step
    float T_default;           // temperature of a primitive whose solve is not finite
    float *Tout;               // [n]
    float *out;                // [n*5] sensible, latent, storage, net radiation, VPD (or null)
    unsigned *status;          // primitives not converged (or null)
};
cudaError_t launch_energy_balance(const EnergyParams &p, cudaStream_t s);
cudaError_t launch_net_radiation(int n, int Bl, const float *flux, float *R, cudaStream_t s);
cudaError_t launch_max_abs_diff(int n, const float *a, const float *b, unsigned *out, cudaStream_t s);

// ---------------------------------------------------------------- BVH build
struct BvhBuffers {
    float4 *rec;        // out: sorted records [n*4]
    float4 *rgen;       // out: origin records [n*4]
    float4 *nodes;      // out: packed nodes [max(n-1,1)*4]
    uint64_t *codes;    // out: sorted Morton codes [n]
    uint32_t *perm;     // out: sorted slot -> original index [n]
    // scratch
    float4 *rec_tmp;    // [n*4]
    float *aabb;        // [n*6]
    float *leafbox;     // [n*6]
    float *nodebox;     // [(n-1)*6]
    float *bounds;      // [16]
    float *partial;     // [nparts*12]
    uint64_t *keys_alt; // [n]
    uint32_t *vals_alt; // [n]
    uint32_t *hist;     // [256*nblk]
    uint32_t *offs;     // [256*nblk]
    uint32_t *scan_tmp; // [scan scratch]
    int32_t *child;     // [2*(n-1)]
    int32_t *parent_int;// [n-1]
    int32_t *parent_leaf;// [n]
    uint32_t *flags;    // [n-1]
    uint32_t *status;   // device error word
};
// Scratch bytes of bvh_build for n primitives (each piece rounded up to 256 B).
constexpr size_t align256c(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t bvh_scratch_bytes_c(int n) {
    size_t nn = (size_t)(n > 1 ? n : 1), ni = (size_t)(n > 1 ? n - 1 : 1);
    size_t nh = 256 * ((nn + 2047) / 2048);
    return align256c(nn * 4 * 16) + align256c(nn * 6 * 4) + align256c(nn * 6 * 4) + align256c(ni * 6 * 4) +
           align256c(16 * 4) + align256c(1024 * 12 * 4) + align256c(nn * 8) + align256c(nn * 4) +
           align256c(nh * 4) + align256c(nh * 4) + align256c((2 * ((nh + 2047) / 2048) + 64) * 4) +
           align256c(2 * ni * 4) + align256c(ni * 4) + align256c(nn * 4) + align256c(ni * 4);
}
size_t bvh_scratch_bytes(int n);
void bvh_carve(BvhBuffers &b, void *scratch, int n);
// Binary BVH over the LBVH's leaf slots by locally-ordered agglomerative clustering (better
// surface-area cost than the Morton split; the 4-wide nodes are collapsed from it).  leafbox:
// [n*6] padded leaf boxes of bvh_build; nodes: [n-1] binary nodes, root 0; n >= 2.
size_t ploc_scratch_bytes(int n);
cudaError_t ploc_build(const float *leafbox, int n, float4 *nodes, void *scratch, cudaStream_t s);
// Compressed 4-wide BVH collapsed from the binary nodes (hrt_bvh4.cu): nodes4 holds
// bvh4_node_capacity(n) nodes of 4 float4, scratch bvh4_scratch_bytes(n); *count_out = the
// highest node index used + 1 (node 1 and the odd tail of some sibling groups are padding).
size_t bvh4_scratch_bytes(int n);
size_t bvh4_node_capacity(int n);
cudaError_t bvh4_build(const float4 *nodes2, int n, float4 *nodes4, void *scratch, uint32_t *status, int *count_out,
                       cudaStream_t s);
// lad: [n] leaf area density of voxels (original order), or null (voxels then hold no leaves).
cudaError_t bvh_build(const float *T, const uint32_t *type, const float *lad, int n, BvhBuffers &b, cudaStream_t s);
constexpr int kSortTile = 2048;

// ---------------------------------------------------------------- passes
cudaError_t launch_direct(const DirectParams &p, int max_blocks, cudaStream_t s);
cudaError_t launch_diffuse(const DiffuseParams &p, int max_blocks, cudaStream_t s);
// Diffuse kernel variants the tuner chooses between: persistent threads over binary nodes
// (PS4 / PS3: 4 or 3 resident blocks per SM), over compressed 4-wide nodes (W4 / W43), or
// one ray per thread over binary nodes (SIMPLE).
enum DiffuseVariant {
    DV_DEFAULT = 0, DV_PS4 = 1, DV_PS3 = 2, DV_SIMPLE = 3, DV_W4 = 4, DV_W43 = 5,
    // lean 4-wide trace (k_diffuse_w4): threads per block x resident blocks per SM, shared
    // stack entries per lane (r: a ring over local memory, l: the bottom entries), ray ids a
    // warp takes per fetch (32 x batch) -- 256 x 4, 8r, 1; 256 x 5, 8r, 1; 256 x 4, 16l, 1;
    // 128 x 8, 8r, 1; 512 x 2, 8r, 1; 256 x 4, 8r, 4; 256 x 4, 8r, 16; 256 x 4, 32l, 1
    DV_W4S4 = 6, DV_W4S5 = 7, DV_W4S4D16 = 8, DV_W4B128 = 9, DV_W4B512 = 10, DV_W4K4 = 11, DV_W4K16 = 12,
    DV_W4S4D32 = 13, DV_LAST = DV_W4S4D32
};
bool is_w4s_variant(int v);
cudaError_t launch_w4s(const DiffuseParams &p, int variant, cudaStream_t s);
cudaError_t launch_w4s_record(const DiffuseParams &p, uint32_t *hits, int variant, cudaStream_t s);
cudaError_t launch_w4s_stats(const DiffuseParams &p, int variant, cudaStream_t s);
// Multi-scene recording launch: p.fetch, p.faces, p.slots / nslots / multi_total set; the
// other scene fields of p are unused.
cudaError_t launch_w4s_multi_record(const DiffuseParams &p, cudaStream_t s);
cudaError_t launch_diffuse_variant(const DiffuseParams &p, int variant, int max_blocks, cudaStream_t s);
// persistent-kernel launchers (hrt_ps_accumulate.cu, hrt_ps_special.cu)
cudaError_t launch_ps_accumulate(const DiffuseParams &p, int variant, cudaStream_t s);
cudaError_t launch_ps_voxels(const DiffuseParams &p, int variant, cudaStream_t s);
cudaError_t launch_ps_stats(const DiffuseParams &p, cudaStream_t s);
// Same launches with per-ray node-visit / primitive-test counting into sc.visits.
cudaError_t launch_direct_stats(const DirectParams &p, int max_blocks, cudaStream_t s);
// variant DV_SIMPLE counts on the binary tree (the structure the host oracle traverses),
// DV_DEFAULT on the tree the default kernel traverses.
cudaError_t launch_diffuse_stats(const DiffuseParams &p, int variant, int max_blocks, cudaStream_t s);
// Launches whose scene holds translucent covers (sc.cover and the gl fields set).
cudaError_t launch_direct_glass(const DirectParams &p, int max_blocks, cudaStream_t s);
cudaError_t launch_diffuse_glass(const DiffuseParams &p, int max_blocks, cudaStream_t s);
cudaError_t launch_trace_rays(const TraceScene &sc, int64_t nrays, const float *o, const float *d, float tmin,
                              float tmax, int anyhit, int32_t *hit, float *t, int32_t *face, cudaStream_t s);
cudaError_t launch_gen_rays(const TraceScene &sc, int kind, uint32_t seed, uint32_t pass, int dimx, int dimy,
                            int face, float dx, float dy, float dz, float *o, float *d, cudaStream_t s);

// ---------------------------------------------------------------- batched sweep
// C = nsun * Bl channels share one scene; channel c = sun * Bl + band.
struct SweepDirectParams {
    TraceScene sc;
    const float *sun_dir;     // [nsun*3] unit directions toward the suns (device)
    int nsun;
    int dimx, dimy;
    uint32_t seed;
    double *G;                // [n*nsun*2] strength sums of unoccluded rays, [p][sun][face]
};
struct GatherParams {
    int n, C, R;              // primitives, channels, rays per primitive and face
    int faces;                // bit 0 top, bit 1 bottom
    const int8_t *twosided;
    const uint32_t *hits;     // [face][n][R] hit codes (prim<<1|face, kMissCode, kLostCode)
    const float *otop, *obot; // [n*C]
    const float *sky;         // [C] isotropic sky flux per channel (0 in scattering passes)
    double *Gt, *Gb;          // [n*C]
};
constexpr uint32_t kMissCode = 0xFFFFFFFFu, kLostCode = 0xFFFFFFFEu;
cudaError_t launch_direct_sweep(const SweepDirectParams &p, int max_blocks, cudaStream_t s);
// Persistent diffuse trace that stores every ray's hit code instead of accumulating.
cudaError_t launch_diffuse_record(const DiffuseParams &p, uint32_t *hits, int variant, cudaStream_t s);
cudaError_t launch_gather(const GatherParams &p, cudaStream_t s);
struct ChannelEpilogue {
    int n, C, Bl;
    const float *rho, *tau;   // [n*Bl]
    const float *flux;        // direct: [C] source flux per channel
    const uint8_t *mask;      // [C] 1 = apply this pass to the channel
    double *rin, *stop, *sbot;
    const double *Gt, *Gb;    // diffuse [n*C]
    const double *Gd;         // direct [n*nsun*2]
    double strength;          // diffuse 1/R
};
cudaError_t launch_epilogue_direct_channels(const ChannelEpilogue &p, cudaStream_t s);
cudaError_t launch_epilogue_diffuse_channels(const ChannelEpilogue &p, cudaStream_t s);
// out = (float)src for channels with mask[c]; optionally src = 0 afterwards (zero != 0)
cudaError_t launch_copy_channels(int n, int C, const uint8_t *mask, double *src_top, double *src_bot, float *otop,
                                 float *obot, int zero, cudaStream_t s);
// one-sided fold of the direct scatter for masked channels, then scatter = 0 for them
cudaError_t launch_fold_channels(int n, int C, const uint8_t *mask, const int8_t *twosided, double *stop,
                                 double *sbot, float *otop, float *obot, cudaStream_t s);

// Epilogues: fold per-face sums into radiation_in / scatter buffers.
struct EpilogueParams {
    int n, Bc, Bl, Bg, S, nsrc_mat;
    const uint8_t *flags;      // [Bg] band flags of this launch (device)
    const float *rho, *tau;    // [Smat*n*Bg]
    double *rin, *stop, *sbot; // [n*Bl]
    const double *Gt, *Gb;     // diffuse: [n*Bl]
    const double *Gd;          // direct: [n*S*2]
    const double *Gcov;        // direct, launches with covers: [n*S*2*Bl] (null: none)
    const float *src_flux;     // direct: [S*Bl]
    double strength;           // diffuse: 1/(dimx*dimy)
};
cudaError_t launch_epilogue_direct(const EpilogueParams &p, cudaStream_t s);
cudaError_t launch_epilogue_diffuse(const EpilogueParams &p, cudaStream_t s);

// Buffer bookkeeping (OptiX8Backend.cpp:1168-1250 semantics).
cudaError_t launch_to_float(const double *a, float *out, size_t n, cudaStream_t s);
cudaError_t launch_fold_onesided(int n, int Bl, const int8_t *twosided, const double *stop, const double *sbot,
                                 double *ftop, double *fbot, cudaStream_t s);
cudaError_t launch_emission(int n, int Bl, const uint8_t *emission, const int32_t *depth, const float *eps,
                            const float *temperature, const int8_t *twosided, double *ftop, double *fbot,
                            cudaStream_t s);
cudaError_t launch_final_flux(size_t nb, const double *rin, const double *stop, const double *sbot, float *out,
                              cudaStream_t s);
// Per-band scattering residual sums into scratch[0 .. 2*Bl): (num, den) pairs, see
// k_residual.  scratch holds 64 + kResidualBlocks * Bl * 2 doubles.
constexpr int kResidualBlocks = 304;
cudaError_t launch_residual(int n, int Bl, const double *area, const double *rin, const double *stop,
                            const double *sbot, double *scratch, cudaStream_t s);

}  // namespace hrt
