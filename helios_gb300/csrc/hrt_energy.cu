// hrt_energy.cu -- surface energy balance: the step after the radiation solve.
//
// Replaces the reference's energy balance kernel (plugins/energybalance/src/
// EnergyBalanceModel.cu:34-125, solveEnergyBalance) and the output fluxes it derives
// (:466-505).  Per primitive, the surface temperature T closes
//   R = Nsides eps sigma T^4 + QH(T) + QL(T) + Qother + storage(T),
// with sensible heat QH = cp gH (T - Ta), latent heat QL = gM lambda (es(T) - ea hs) / P through
// the series conductance gM of the boundary layer and the stomata, and storage C (T - Tprev) / dt.
// The root is found by the secant method from (Tprev, 400 K), relative step 1e-4, at most 100
// steps, as the reference does, so the temperatures agree with it step for step.
#include <cuda_runtime.h>

#include <cstdint>

#include "hrt_internal.h"

namespace hrt {

namespace {

constexpr float kCpAirMol = 29.25f;      // J/mol/K
constexpr float kLambdaMol = 44000.f;    // J/mol
constexpr float kSigmaEB = 5.67e-8f;     // the energy balance's Stefan-Boltzmann constant

__device__ __forceinline__ float moisture_gm(float gH, float gS, float s) {
    if (gH == 0.f || gS == 0.f) return 0.f;
    return 1.08f * gH * gS * (s / (1.08f * gH + gS * s) + (1.f - s) / (1.08f * gH + gS * (1.f - s)));
}

// Residual of the balance at T (the reference's evaluateEnergyBalance).
__device__ __forceinline__ float eb_residual(float T, const EnergyParams &P, int p, float Tprev) {
    const float Rout = (float)P.nsides[p] * P.eps[p] * kSigmaEB * T * T * T * T;
    const float QH = kCpAirMol * P.gH[p] * (T - P.Ta[p]);
    const float es = 611.0f * expf(17.502f * (T - 273.f) / (T - 273.f + 240.97f));
    const float QL = moisture_gm(P.gH[p], P.gS[p], P.sided[p]) * kLambdaMol * (es - P.ea[p] * P.hs[p]) / P.press[p];
    const float storage = P.dt > 0.f ? P.cap[p] * (T - Tprev) / P.dt : 0.f;
    return P.R[p] - Rout - QH - QL - P.Qother[p] - storage;
}

__global__ void k_energy_balance(const EnergyParams P) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const float Tprev = P.Tin[p];
    float T0 = Tprev, T1 = 400.f;
    if (T1 == T0) T1 = T0 + 100.f;
    float T = T0;
    float r0 = eb_residual(T0, P, p, Tprev), r1 = eb_residual(T1, P, p, Tprev);
    float err = 100.f;
    for (int it = 0; it < 100 && err > 1e-4f; ++it) {
        if (r0 == r1) {
            err = 0.f;
            break;
        }
        T = fabsf((T1 * r0 - T0 * r1) / (r0 - r1));
        const float r = eb_residual(T, P, p, Tprev);
        err = fabsf(T - T0) / fabsf(T0);
        r1 = r0;
        r0 = r;
        T1 = T0;
        T0 = T;
    }
    if (!isfinite(T)) T = P.T_default;
    if (err > 1e-4f && P.status) atomicAdd(P.status, 1u);  // not converged (counted)
    P.Tout[p] = T;
    if (P.out) {
        const float gH = P.gH[p];
        const float es = 611.0f * expf(17.502f * (T - 273.15f) / (T - 273.15f + 240.97f));
        float *o = P.out + 5 * (size_t)p;
        o[0] = kCpAirMol * gH * (T - P.Ta[p]);                                                  // sensible
        o[1] = kLambdaMol * moisture_gm(gH, P.gS[p], P.sided[p]) * (es - P.ea[p]) / P.press[p];  // latent
        o[2] = P.dt > 0.f ? P.cap[p] * (T - Tprev) / P.dt : 0.f;                                // storage
        o[3] = P.R[p] - (float)P.nsides[p] * P.eps[p] * kSigmaEB * T * T * T * T;              // net radiation
        o[4] = (es - P.ea[p]) / P.press[p];                                                     // vapour pressure deficit
    }
}

// R[p] = sum over the bands of the solve's flux [n*Bl]
__global__ void k_net_radiation(int n, int Bl, const float *__restrict__ flux, float *__restrict__ R) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float s = 0.f;
    for (int b = 0; b < Bl; ++b) s += flux[(size_t)p * Bl + b];
    R[p] = s;
}

// largest |a - b| (non-negative floats order as their bit patterns)
__global__ void k_max_abs_diff(int n, const float *__restrict__ a, const float *__restrict__ b, unsigned *out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    float d = 0.f;
    if (p < n) d = fabsf(a[p] - b[p]);
    if (!(d >= 0.f)) d = __int_as_float(0x7f800000);  // NaN counts as not converged
    for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_down_sync(0xffffffffu, d, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(d));
}

}  // namespace

cudaError_t launch_energy_balance(const EnergyParams &p, cudaStream_t s) {
    if (p.n <= 0) return cudaSuccess;
    k_energy_balance<<<(p.n + 127) / 128, 128, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_net_radiation(int n, int Bl, const float *flux, float *R, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_net_radiation<<<(n + 255) / 256, 256, 0, s>>>(n, Bl, flux, R);
    return cudaGetLastError();
}

cudaError_t launch_max_abs_diff(int n, const float *a, const float *b, unsigned *out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_max_abs_diff<<<(n + 255) / 256, 256, 0, s>>>(n, a, b, out);
    return cudaGetLastError();
}

}  // namespace hrt
