// Hosek-Wilkie analytic sky texture (renderer/gpu_kernels/analytic_sky_kernels.cu:16-276,
// itself a device port of ext/hosek_wilkie_2013/ArHosekSkyModel.c v1.4a). The per-band
// model states are computed on the host by the published model and passed in as plain
// floats with the model's solar tables; this file evaluates the radiance functions per texel,
// including the direct solar radiance at each disc texel's own elevation.
#include <memory>

#include "vpt_ctx.h"
#include "vpt_scene.cuh"

namespace vpt {
namespace {

constexpr int kBands = 16;
constexpr int kStateFloats = 122;  // configs[11][9], radiances[11], ecf_sky[11], solar_radius
constexpr int kChannels = 11;      // 320, 360, ..., 720 nm
constexpr int kPieces = 45, kOrder = 4;
constexpr int kSolarTable = kPieces * kOrder;

struct SkyBand {
    float configs[11][9];
    float radiances[11];
    float ecf_sky[11];
    float solar_radius;
};
struct SkyConst {
    SkyBand band[kBands];
    float xs[kBands], ys[kBands], zs[kBands], center_wl[kBands];
    float integral_cmf;
    // Solar disc: weight of the upper of the two turbidities around the requested one, the
    // model's piecewise-cubic direct-radiance tables of both per channel (coefficients of a piece
    // highest order first, as the model stores them) and its limb-darkening coefficients.
    float turb_frac;
    float solar[kChannels][2][kSolarTable];
    float limb[kChannels][6];
};
__constant__ SkyConst c_sky;

// analytic_sky_kernels.cu:16-27.
__device__ __forceinline__ float radiance_internal(const float* cfg, float theta, float gamma) {
    const float exp_m = expf(cfg[4] * gamma);
    const float ray_m = cosf(gamma) * cosf(gamma);
    const float mie_m = (1.0f + cosf(gamma) * cosf(gamma)) /
                        powf((1.0f + cfg[8] * cfg[8] - 2.0f * cfg[8] * cosf(gamma)), 1.5f);
    const float zenith = sqrtf(cosf(theta));
    return (1.0f + cfg[0] * expf(cfg[1] / (cosf(theta) + 0.01f))) *
           (cfg[2] + cfg[3] * exp_m + cfg[5] * ray_m + cfg[6] * mie_m + cfg[7] * zenith);
}

// analytic_sky_kernels.cu:29-66.
__device__ __forceinline__ float sky_radiance(const SkyBand& s, float theta, float gamma, float wavelength) {
    int low_wl = static_cast<int>((wavelength - 320.0f) / 40.0f);
    if (low_wl < 0 || low_wl >= 11) return 0.0f;
    float interp = fmodf((wavelength - 320.0f) / 40.0f, 1.0f);
    float val_low = radiance_internal(s.configs[low_wl], theta, gamma) * s.radiances[low_wl] * s.ecf_sky[low_wl];
    if (interp < 1e-6f) return val_low;
    float result = (1.0f - interp) * val_low;
    if (low_wl + 1 < 11)
        result += interp * radiance_internal(s.configs[low_wl + 1], theta, gamma) * s.radiances[low_wl + 1] *
                  s.ecf_sky[low_wl + 1];
    return result;
}

// analytic_sky_kernels.cu:69-97: the direct solar radiance of one channel at one of the two
// turbidities (slot 0: lower, 1: upper), a cubic in the elevation on 45 pieces.
__device__ __forceinline__ float sr_internal(int slot, int wl, float elevation) {
    int pos = static_cast<int>(powf(2.0f * elevation / kPi, 1.0f / 3.0f) * kPieces);
    if (pos > kPieces - 1) pos = kPieces - 1;
    const float break_x = powf(static_cast<float>(pos) / static_cast<float>(kPieces), 3.0f) * (kPi * 0.5f);
    const float* coefs = &c_sky.solar[wl][slot][kOrder * (pos + 1) - 1];
    float res = 0.0f;
    const float x = elevation - break_x;
    float x_exp = 1.0f;
    for (int i = 0; i < kOrder; ++i) {
        res += x_exp * *coefs--;
        x_exp *= x;
    }
    return res;  // times the sun's emission correction, 1 for this model state
}

// analytic_sky_kernels.cu:99-184: interpolated between turbidities and channels, limb-darkened.
__device__ __forceinline__ float solar_direct(const SkyBand& s, float wavelength, float elevation, float gamma) {
    const float tf = c_sky.turb_frac;
    int wl_low = static_cast<int>((wavelength - 320.0f) / 40.0f);
    float wl_frac = fmodf(wavelength, 40.0f) / 40.0f;
    if (wl_low == 10) {
        wl_low = 9;
        wl_frac = 1.0f;
    }
    const float direct =
        (1.0f - tf) * ((1.0f - wl_frac) * sr_internal(0, wl_low, elevation) + wl_frac * sr_internal(0, wl_low + 1, elevation)) +
        tf * ((1.0f - wl_frac) * sr_internal(1, wl_low, elevation) + wl_frac * sr_internal(1, wl_low + 1, elevation));
    float ld[6];
    for (int i = 0; i < 6; ++i) ld[i] = (1.0f - wl_frac) * c_sky.limb[wl_low][i] + wl_frac * c_sky.limb[wl_low + 1][i];
    const float sol_rad_sin = sinf(s.solar_radius);
    const float ar2 = 1 / (sol_rad_sin * sol_rad_sin);
    const float singamma = sinf(gamma);
    float sc2 = 1.0f - ar2 * singamma * singamma;
    if (sc2 < 0.0f) sc2 = 0.0f;
    const float c = sqrtf(sc2);
    const float darkening = ld[0] + ld[1] * c + ld[2] * powf(c, 2.0f) + ld[3] * powf(c, 3.0f) + ld[4] * powf(c, 4.0f) +
                            ld[5] * powf(c, 5.0f);
    return direct * darkening;
}

// analytic_sky_kernels.cu:194-214: direct radiance at the texel's elevation plus the sky.
__device__ __forceinline__ float solar_radiance(const SkyBand& s, float theta, float gamma, float wavelength) {
    return solar_direct(s, wavelength, (kPi / 2.0f) - theta, gamma) + sky_radiance(s, theta, gamma, wavelength);
}

// basic_types.h:3114-3160 (HSV conversions).
__device__ __forceinline__ void rgb_to_hsv(float r, float g, float b, float* h, float* s, float* v) {
    float mn = fminf(fminf(r, g), b);
    float mx = fmaxf(fmaxf(r, g), b);
    *v = mx;
    float delta = mx - mn;
    if (delta < 1e-5f || mx == 0.0f) {
        *h = 0.0f;
        *s = 0.0f;
        return;
    }
    *s = delta / mx;
    if (r >= mx)
        *h = (g - b) / delta;
    else if (g >= mx)
        *h = 2.0f + (b - r) / delta;
    else
        *h = 4.0f + (r - g) / delta;
    *h /= 6;
    *h = fmodf(*h + 1.0f, 1.0f);
}
__device__ __forceinline__ RGB hsv_to_rgb(float h, float s, float v) {
    if (s == 0) return rgb(v, v, v);
    h = h - floorf(h);
    int hi = static_cast<int>(h * 6);
    float f = h * 6 - hi;
    float m = v * (1 - s);
    float n = v * (1 - s * f);
    float k = v * (1 - s * (1 - f));
    switch (hi) {
    case 0: return rgb(v, k, m);
    case 1: return rgb(n, v, m);
    case 2: return rgb(m, v, k);
    case 3: return rgb(m, n, v);
    case 4: return rgb(k, m, v);
    case 5: return rgb(v, m, n);
    default: return rgb(0, 0, 0);
    }
}

// analytic_sky_kernels.cu:220-276.
__global__ void sky_kernel(float4* __restrict__ out, int w, int h, float sx, float sy, float sz, int include_disc) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    float theta = kPi * (y + 0.5f) / h;
    float phi = 2 * kPi * (x + 0.5f) / w;
    float m_theta = theta;
    bool lower = theta >= 0.5f * kPi;
    if (lower) m_theta = kPi - theta;
    V3 view = from_polar_yup(phi, m_theta);
    float gamma = acosf(fminf(fmaxf(dot(view, v3(sx, sy, sz)), -1.0f), 1.0f));
    float X = 0, Y = 0, Z = 0;
    for (int b = 0; b < kBands; ++b) {
        const SkyBand& s = c_sky.band[b];
        float wl = fminf(fmaxf(c_sky.center_wl[b], 320.0f), 720.0f);
        float value;
        if (include_disc && gamma < s.solar_radius && !lower)
            value = solar_radiance(s, m_theta, gamma, wl);
        else
            value = sky_radiance(s, m_theta, gamma, wl);
        X += c_sky.xs[b] * value;
        Y += c_sky.ys[b] * value;
        Z += c_sky.zs[b] * value;
    }
    X /= c_sky.integral_cmf;
    Y /= c_sky.integral_cmf;
    Z /= c_sky.integral_cmf;
    // basic_types.h:3000-3010 (XYZ -> linear sRGB).
    RGB c = rgb(3.2404542f * X + -1.5371385f * Y + -0.4985314f * Z, -0.9692660f * X + 1.8760108f * Y + 0.0415560f * Z,
                0.0556434f * X + -0.2040259f * Y + 1.0572252f * Z);
    float max_v = fmaxf(c.r, fmaxf(c.g, c.b));
    c = rdiv(c, max_v);
    float hh, ss, vv;
    rgb_to_hsv(c.r, c.g, c.b, &hh, &ss, &vv);
    float diff_hue = fmodf(hh - 2.0f / 3 + 1.0f, 1.0f);
    float diff_angle = 2 * kPi * diff_hue;
    float t_s = ss * powf(0.5f * (1 + cosf(diff_angle)), 1.0f);
    ss = (1 - t_s) * ss + t_s * 1.0f;
    c = max_v * hsv_to_rgb(hh, ss, 1.0f);
    if (lower) {
        // common_shared.h:233-235 lerp = (1 - t) * v0 + t * v1.
        float sea_b = (1 - sy) * 0.01f + sy * 0.1f;
        RGB sea = 0.5f * rgb(0.01f, 0.01f, sea_b);
        float t = powf(cosf(m_theta), 1 / 5.0f);
        c = (1 - t) * c + t * sea;
    }
    out[static_cast<int64_t>(y) * w + x] = make_float4(c.r, c.g, c.b, 0.0f);
}

}  // namespace

int generate_sky_texture(float4* out, int w, int h, const float* states, const float* solar, const float* cmf,
                         const float sun_dir[3], int include_disc) {
    std::unique_ptr<SkyConst> owner(new SkyConst);  // 24 KB: kept off the stack
    SkyConst& sc = *owner;
    for (int b = 0; b < kBands; ++b) {
        const float* st = states + b * kStateFloats;
        SkyBand& d = sc.band[b];
        for (int i = 0; i < 11; ++i)
            for (int j = 0; j < 9; ++j) d.configs[i][j] = st[i * 9 + j];
        for (int i = 0; i < 11; ++i) d.radiances[i] = st[99 + i];
        for (int i = 0; i < 11; ++i) d.ecf_sky[i] = st[110 + i];
        d.solar_radius = st[121];
    }
    sc.turb_frac = solar[0];
    const float* tables = solar + 1;
    for (int wl = 0; wl < kChannels; ++wl)
        for (int t = 0; t < 2; ++t)
            for (int i = 0; i < kSolarTable; ++i) sc.solar[wl][t][i] = tables[(wl * 2 + t) * kSolarTable + i];
    const float* limb = tables + kChannels * 2 * kSolarTable;
    for (int wl = 0; wl < kChannels; ++wl)
        for (int i = 0; i < 6; ++i) sc.limb[wl][i] = limb[wl * 6 + i];
    for (int b = 0; b < kBands; ++b) {
        sc.xs[b] = cmf[b];
        sc.ys[b] = cmf[16 + b];
        sc.zs[b] = cmf[32 + b];
        sc.center_wl[b] = cmf[48 + b];
    }
    sc.integral_cmf = cmf[64];
    if (cudaMemcpyToSymbol(c_sky, &sc, sizeof(sc)) != cudaSuccess)
        return ctx_set_error(-2, "cudaMemcpyToSymbol(sky constants) failed");
    dim3 block(16, 8), grid((w + 15) / 16, (h + 7) / 8);
    sky_kernel<<<grid, block>>>(out, w, h, sun_dir[0], sun_dir[1], sun_dir[2], include_disc);
    if (cudaGetLastError() != cudaSuccess) return ctx_set_error(-2, "sky kernel launch failed");
    return 0;
}

}  // namespace vpt
