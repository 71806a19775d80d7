/*
 * ORACLE (test infrastructure only) — CPU generator of the seeded synthetic volumes.
 *
 * The reference renders NanoVDB assets (renderer/renderer_scene.cpp:491-537); the GB300
 * workloads replace them with seeded fBm value noise defined by this project (integer lattice
 * hash, quintic fade, octaves summed with gain and lacunarity, min-max remap to [0, 1], optional
 * threshold for sparse clouds, optional union of two clouds by max). This file states that
 * generator on the host so that tests and the CPU baseline build their volumes without the
 * product library. Every float operation is a single IEEE operation in the same order as the
 * device generator (which is compiled without FMA contraction), so the two agree bit for bit.
 */
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

inline float lattice_value(int ix, int iy, int iz, uint32_t seed) {
    uint32_t h = seed * 0x9E3779B1u;
    const int c[3] = {ix, iy, iz};
    for (int a = 0; a < 3; ++a) {
        h ^= static_cast<uint32_t>(c[a]) * 0x85EBCA77u;
        h = rotl32(h, 13) * 0xC2B2AE3Du;
    }
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    h *= 0x846ca68bu;
    h ^= h >> 16;
    return static_cast<float>(h >> 8) * (1.0f / 16777216.0f);
}

inline float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
inline float lerp(float a, float b, float w) { return a + w * (b - a); }

float value_noise(float x, float y, float z, uint32_t seed) {
    float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    int ix = static_cast<int>(fx), iy = static_cast<int>(fy), iz = static_cast<int>(fz);
    float wx = fade(x - fx), wy = fade(y - fy), wz = fade(z - fz);
    float c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 2; ++d) c[a][b][d] = lattice_value(ix + a, iy + b, iz + d, seed);
    float x00 = lerp(c[0][0][0], c[1][0][0], wx);
    float x10 = lerp(c[0][1][0], c[1][1][0], wx);
    float x01 = lerp(c[0][0][1], c[1][0][1], wx);
    float x11 = lerp(c[0][1][1], c[1][1][1], wx);
    float y0 = lerp(x00, x10, wy);
    float y1 = lerp(x01, x11, wy);
    return lerp(y0, y1, wz);
}

// One cloud: raw fBm, min-max remap, optional threshold. Layout x-major (x slowest, z fastest).
void fbm_cloud(float* out, int n, uint32_t seed, int octaves, float lacunarity, float gain, float base_frequency,
               float threshold) {
    const int64_t total = static_cast<int64_t>(n) * n * n;
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < total; ++idx) {
        int z = static_cast<int>(idx % n);
        int y = static_cast<int>((idx / n) % n);
        int x = static_cast<int>(idx / (static_cast<int64_t>(n) * n));
        float fn = static_cast<float>(n);
        float px = (static_cast<float>(x) + 0.5f) / fn, py = (static_cast<float>(y) + 0.5f) / fn,
              pz = (static_cast<float>(z) + 0.5f) / fn;
        float freq = base_frequency, amp = 1.0f, sum = 0.0f, norm = 0.0f;
        for (int o = 0; o < octaves; ++o) {
            float v = value_noise(px * freq, py * freq, pz * freq, seed + 1013u * static_cast<uint32_t>(o));
            float term = amp * v;
            sum = sum + term;
            norm += amp;
            amp *= gain;
            freq *= lacunarity;
        }
        out[idx] = sum / norm;
    }
    float lo = FLT_MAX, hi = 0.0f;
#pragma omp parallel for reduction(min : lo) reduction(max : hi) schedule(static)
    for (int64_t i = 0; i < total; ++i) {
        lo = std::min(lo, out[i]);
        hi = std::max(hi, out[i]);
    }
    float scale = hi > lo ? 1.0f / (hi - lo) : 0.0f;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < total; ++i) {
        float r = (out[i] - lo) * scale;
        if (threshold > 0.0f) r = r > threshold ? (r - threshold) / (1.0f - threshold) : 0.0f;
        out[i] = r;
    }
}

}  // namespace

extern "C" {

// Dense n^3 fBm volume (values in [0, 1]); `union_seed` >= 0 adds a second cloud of the same
// parameters with that seed, unioned by max. `scratch` (n^3 floats) is needed only for a union.
void orc_fbm_volume(int32_t n, uint32_t seed, int64_t union_seed, int32_t octaves, float lacunarity, float gain,
                    float base_frequency, float threshold, float* out, float* scratch) {
    fbm_cloud(out, n, seed, octaves, lacunarity, gain, base_frequency, threshold);
    if (union_seed < 0 || scratch == nullptr) return;
    fbm_cloud(scratch, n, static_cast<uint32_t>(union_seed), octaves, lacunarity, gain, base_frequency, threshold);
    const int64_t total = static_cast<int64_t>(n) * n * n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < total; ++i) out[i] = std::max(out[i], scratch[i]);
}

}  // extern "C"
