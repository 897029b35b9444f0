// Host check of the ray-id decoding by multiplication (FastDiv in hrt_device.cuh): every
// divisor against plain division, over edge and pseudo-random numerators.  Prints the number
// of mismatches and exits non-zero on any.
#include <cstdint>
#include <cstdio>

#include "hrt_device.cuh"

static uint64_t rng_state = 0x9E3779B97F4A7C15ull;
static uint32_t next32() {  // SplitMix64, high half
    uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return (uint32_t)((z ^ (z >> 31)) >> 32);
}

static long check(uint32_t d) {
    const hrt::FastDiv f = hrt::make_fastdiv(d);
    long bad = 0;
    const uint32_t edge[] = {0u, 1u, d - 1u, d, d + 1u, 2u * d - 1u, 2u * d, 0x7FFFFFFFu, 0x80000000u,
                             0xFFFFFFFFu, 0xFFFFFFFFu - d, (0xFFFFFFFFu / d) * d, (0xFFFFFFFFu / d) * d - 1u};
    for (uint32_t n : edge)
        if (hrt::fast_div(n, f) != n / d) ++bad;
    for (int i = 0; i < 256; ++i) {
        const uint32_t n = next32();
        if (hrt::fast_div(n, f) != n / d) ++bad;
    }
    return bad;
}

int main() {
    long bad = 0, ndiv = 0;
    for (uint32_t d = 1; d <= 70000; ++d, ++ndiv) bad += check(d);   // every ray count and stratum count in use
    for (int k = 1; k < 32; ++k, ndiv += 3) bad += check(1u << k) + check((1u << k) - 1u) + check((1u << k) + 1u);
    for (int i = 0; i < 20000; ++i, ++ndiv) bad += check(next32() | 1u);
    bad += check(0xFFFFFFFFu);
    std::printf("divisors %ld mismatches %ld\n", ndiv + 1, bad);
    return bad ? 1 : 0;
}
