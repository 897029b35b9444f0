// hrt_camera.cu -- camera and pixel-label rays.
//
// Replaces the reference's camera programs (plugins/radiation/src/optix8/OptiX8DeviceCode.cu):
//   __raygen__camera        :1665-1738 -> k_camera (ray generation)
//   __closesthit__camera    :1007-1170 -> cam_value (hit: radiation_out + sources in front)
//   __miss__camera          :673-741   -> cam_value (miss: sources, solar disk, sky)
//   __raygen__pixel_label   :1744-1812 -> k_pixel_label
//   __closesthit__pixel_label :1176-1199, __miss__pixel_label :743-748
// A camera ray of pixel (ii, jj), sample s draws its sub-pixel offset and lens point from
// Philox counter (pixel, s, kCamCounter, 0) keyed by (seed, camera id), so an image does not
// depend on how it is tiled.  The samples of a pixel are consecutive ray ids, so a warp sums
// them with the segmented shuffle reduction before one FP64 atomic per pixel and band.
#include "hrt_trace.cuh"

namespace hrt {

namespace {

constexpr uint32_t kCamCounter = 0xCA3E0001u;
constexpr float kPiF = 3.14159265358979323846f;

__device__ __forceinline__ f3 mrot(const float *M, f3 v) {
    return mk((M[0] * v.x + M[1] * v.y) + M[2] * v.z, (M[3] * v.x + M[4] * v.y) + M[5] * v.z,
              (M[6] * v.x + M[7] * v.y) + M[8] * v.z);
}

// Ray of pixel (ii, jj), sample smp; centre: through the pixel centre and the lens centre.
__device__ __forceinline__ void camera_ray(const CameraParams &P, uint32_t ii, uint32_t jj, uint32_t smp, bool centre,
                                           f3 *o, f3 *d) {
    float rx = 0.5f, ry = 0.5f, lx = 0.f, ly = 0.f;
    if (!centre) {
        const u4 u = philox(jj * (uint32_t)P.W + ii, smp, kCamCounter, 0u, P.seed, P.cam_id);
        rx = u01(u.a);
        ry = u01(u.b);
        if (P.lens > 0.f) concentric(u01(u.c), u01(u.d), &lx, &ly);
    }
    const float spy = -0.5f + ((float)ii + rx) / (float)P.W;
    const float spz = (0.5f - ((float)jj + ry) / (float)P.H) * P.inv_aspect;
    const f3 p = mk(P.focal, spy / P.viewplane * P.focal, spz / P.viewplane * P.focal);
    const f3 org = mk(0.f, 0.5f * lx * P.lens, 0.5f * ly * P.lens);
    *o = add(mrot(P.M, org), mk(P.pos[0], P.pos[1], P.pos[2]));
    *d = normalize(mrot(P.M, sub(p, org)));
}

// Radiance of a sphere, rectangle or disk source seen along (o, d) before distance tlim
// (front faces of rectangles and disks; OptiX8DeviceCode.cu:249-309, 1049-1126).
__device__ __forceinline__ float source_radiance(const SourceDev &sr, float flux, f3 o, f3 d, float tlim) {
    const f3 c = mk(sr.pos[0], sr.pos[1], sr.pos[2]);
    if (sr.type == 1) {
        const float r = 0.5f * sr.w0;
        const f3 oc = sub(o, c);
        const float b = dot(oc, d), cc = dot(oc, oc) - r * r, disc = b * b - cc;
        if (disc < 0.f) return 0.f;
        const float t = -b - sqrtf(disc);
        if (!(t > 0.f && t < tlim)) return 0.f;
        return flux / (4.f * kPiF * r * r) / kPiF;
    }
    if (sr.type == 3 || sr.type == 4) {
        const float *R = sr.R;
        const f3 n = mk(R[2], R[5], R[8]);
        const float den = dot(d, n);
        if (!(den < -1e-6f)) return 0.f;
        const float t = dot(sub(c, o), n) / den;
        if (!(t > 0.f && t < tlim)) return 0.f;
        const f3 hp = sub(add(o, scl(d, t)), c);
        float area;
        if (sr.type == 3) {
            const float lx = (R[0] * hp.x + R[3] * hp.y) + R[6] * hp.z;
            const float ly = (R[1] * hp.x + R[4] * hp.y) + R[7] * hp.z;
            if (fabsf(lx) > 0.5f * sr.w0 || fabsf(ly) > 0.5f * sr.w1) return 0.f;
            area = sr.w0 * sr.w1;
        } else {
            if (dot(hp, hp) > sr.w0 * sr.w0) return 0.f;
            area = kPiF * sr.w0 * sr.w0;
        }
        return flux / area * (-den) / kPiF;
    }
    return 0.f;
}

// Radiance a camera ray adds to its pixel in band b: on a hit, strength x the hit face's
// radiation_out plus the sources in front of the hit, over pi (as the reference's closest-hit
// program divides); on a miss, the sources, the solar disk or the sky, and the isotropic sky
// flux of emission bands.
__device__ float cam_value(const CameraParams &P, const Hit &h, f3 ol, f3 d, int b, float strength) {
    if (h.prim != 0xFFFFFFFFu) {
        const size_t ih = (size_t)h.prim * P.Bl + b;
        float val = strength * __ldg((h.face ? P.otop : P.obot) + ih);
        for (int k = 0; k < P.S; ++k) {
            const float fl = P.src_flux[k * P.Bl + b];
            if (!(fl > 0.f)) continue;
            const float r = source_radiance(P.src[k], fl, ol, d, h.t);
            if (r > 0.f) val += r * strength;
        }
        return val / kPiF;
    }
    float rad = 0.f;
    const float inf = __int_as_float(0x7f800000);
    for (int k = 0; k < P.S; ++k) {
        const float fl = P.src_flux[k * P.Bl + b];
        if (!(fl > 0.f)) continue;
        const int ty = P.src[k].type;
        if (ty == 0 || ty == 2) {
            if (P.disk_rad && P.disk_rad[b] > 0.f && dot(d, mk(P.sun[0], P.sun[1], P.sun[2])) >= P.disk_cos)
                rad += P.disk_rad[b];
        } else {
            rad += source_radiance(P.src[k], fl, ol, d, inf);
        }
    }
    if (rad <= 0.f && P.sky_rad && P.sky_rad[b] > 0.f) rad = P.sky_rad[b] * (float)sky_fd(d, P.sky, b);
    if (P.emission && P.emission[b] && P.dflux && P.dflux[b] > 0.f) rad += P.dflux[b] / kPiF;
    return rad > 0.f ? rad * strength : 0.f;
}

// W4: camera rays over the compressed 4-wide nodes (sc.nodes4 set), else the binary nodes; the
// closest hit does not depend on the tree.
template <int NB, bool W4>
__global__ void __launch_bounds__(kBlock) k_camera(const CameraParams P) {
    const uint32_t aa = (uint32_t)P.aa;
    const uint32_t total = (uint32_t)(P.tw * P.th) * aa;
    const uint32_t stride = gridDim.x * blockDim.x;
    const float strength = 1.0f / (float)P.aa;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total; base += stride) {
        const uint32_t id = base + (threadIdx.x & 31);
        const bool active = id < total;
        uint32_t q = 0xFFFFFFFFu;
        double v[NB];
#pragma unroll
        for (int j = 0; j < NB; ++j) v[j] = 0.0;
        if (active) {
            const uint32_t t = id / aa, smp = id % aa;
            const uint32_t ii = (uint32_t)P.ox + t % (uint32_t)P.tw, jj = (uint32_t)P.oy + t / (uint32_t)P.tw;
            q = jj * (uint32_t)P.W + ii;
            f3 o, d, ol;
            camera_ray(P, ii, jj, smp, false, &o, &d);
            const Hit h = trace_full<false, W4>(P.sc, o, d, 1e-5f, 1e30f, false,
                                                VoxKey{q, smp, 0x40000000u, P.seed, P.cam_id}, nullptr, nullptr, &ol);
            if (h.prim != kLost) {
#pragma unroll
                for (int j = 0; j < NB; ++j)
                    if (j < P.Bl) v[j] = (double)cam_value(P, h, ol, d, j, strength);
            }
        }
        count_rays(P.sc, active);
        warp_segment_add<NB>(q, v, P.Bl, P.pix, P.Bl);
    }
}

template <bool W4>
__global__ void k_pixel_label(const CameraParams P) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint32_t)(P.tw * P.th)) return;
    const uint32_t ii = (uint32_t)P.ox + t % (uint32_t)P.tw, jj = (uint32_t)P.oy + t / (uint32_t)P.tw;
    const uint32_t q = jj * (uint32_t)P.W + ii;
    f3 o, d, ol;
    camera_ray(P, ii, jj, 0u, true, &o, &d);
    const Hit h = trace_full<false, W4>(P.sc, o, d, 1e-5f, 1e30f, false,
                                        VoxKey{q, 0xFFFFFFFFu, 0x40000000u, P.seed, P.cam_id}, nullptr, nullptr, &ol);
    if (h.prim == 0xFFFFFFFFu) {
        P.labels[q] = 0u;
        P.depths[q] = -1.f;
    } else if (h.prim != kLost) {
        P.labels[q] = h.prim + 1u;
        P.depths[q] = fabsf(dot(mk(P.M[0], P.M[3], P.M[6]), d)) * h.t;
    }
}

__global__ void k_add(double *__restrict__ dst, const double *__restrict__ src, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] += src[i];
}

}  // namespace

cudaError_t launch_camera(const CameraParams &p, int max_blocks, cudaStream_t s) {
    const long long total = (long long)p.tw * p.th * p.aa;
    if (total <= 0 || p.Bl <= 0) return cudaSuccess;
    long long nb = (total + kBlock - 1) / kBlock;
    if (nb > max_blocks) nb = max_blocks;
    const bool w4 = p.sc.nodes4 != nullptr;
    if (p.Bl <= 1) w4 ? k_camera<1, true><<<(unsigned)nb, kBlock, 0, s>>>(p) : k_camera<1, false><<<(unsigned)nb, kBlock, 0, s>>>(p);
    else if (p.Bl <= 4) w4 ? k_camera<4, true><<<(unsigned)nb, kBlock, 0, s>>>(p) : k_camera<4, false><<<(unsigned)nb, kBlock, 0, s>>>(p);
    else if (p.Bl <= 16) w4 ? k_camera<16, true><<<(unsigned)nb, kBlock, 0, s>>>(p) : k_camera<16, false><<<(unsigned)nb, kBlock, 0, s>>>(p);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_pixel_labels(const CameraParams &p, cudaStream_t s) {
    const long long total = (long long)p.tw * p.th;
    if (total <= 0) return cudaSuccess;
    if (p.sc.nodes4) k_pixel_label<true><<<(unsigned)((total + 127) / 128), 128, 0, s>>>(p);
    else k_pixel_label<false><<<(unsigned)((total + 127) / 128), 128, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_add(double *dst, const double *src, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dst, src, n);
    return cudaGetLastError();
}

void camera_rotation(float zenith, float azimuth, float M[9]) {
    const double th = -0.5 * M_PI + (double)zenith, ph = 0.5 * M_PI - (double)azimuth;
    const double st = std::sin(th), ct = std::cos(th), sp = std::sin(ph), cp = std::cos(ph);
    const double m[9] = {cp * ct, -sp, cp * st, sp * ct, cp, sp * st, -st, 0.0, ct};
    for (int i = 0; i < 9; ++i) M[i] = (float)m[i];
}

}  // namespace hrt
