// Output of the accumulated image: the reference's tone-map kernel fused with the 8-bit sRGB
// conversion its image saver runs on the host, so one pass over the mean image yields the
// RGBA8 frame the headless loop writes to "%03u.png".
//
// applyToneMap (renderer/gpu_kernels/post_process_kernels.cu:10-41): every channel of the
// running mean raised to 1/0.6, then scaled by (1 - exp(-brightness * lum)) / lum (lum = the
// Rec.709 luminance, basic_types.h:2981-2986; brightness is 1 in the reference). saveImage
// (common/common_host.cpp:517-568) as renderer_main.cpp:1490-1495 configures it: no second tone
// map, negative channels clamped to 0, sRGB_gamma_s (basic_types.h:3181-3188) per channel,
// min(uint(v * 255), 255) per byte, alpha overridden to 1 (255). This unit is compiled without
// multiply-add contraction so the arithmetic follows the written operation order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/rtc8_vpt.h"
#include "vpt_ctx.h"

namespace vpt {
namespace {

__device__ __forceinline__ uint32_t to_byte(float v) {
    // static_cast<uint32_t>(v * 255) clamped to 255; NaN and negative values give 0, +inf 255.
    const float x = v * 255.0f;
    if (!(x > 0.0f)) return 0u;
    if (x >= 255.0f) return 255u;
    return static_cast<uint32_t>(x);
}

__device__ __forceinline__ float srgb_gamma(float v) {
    if (v <= 0.0031308f) return 12.92f * v;
    return 1.055f * powf(v, static_cast<float>(1 / 2.4)) - 0.055f;
}

__global__ void tonemap_kernel(const float* __restrict__ mean, int width, int height, float brightness,
                               uint32_t flags, float4* __restrict__ out_f32, uint32_t* __restrict__ out_rgba8) {
    const int64_t n = static_cast<int64_t>(width) * height;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        constexpr float kGamma = 1.0f / 0.6f;
        float r = powf(mean[3 * i], kGamma), g = powf(mean[3 * i + 1], kGamma), b = powf(mean[3 * i + 2], kGamma);
        const float lum = 0.2126729f * r + 0.7151522f * g + 0.0721750f * b;
        if (lum > 0.0f) {
            const float lum_t = 1 - expf(-brightness * lum);
            const float s = lum_t / lum;
            r *= s;
            g *= s;
            b *= s;
        }
        if (out_f32) out_f32[i] = make_float4(r, g, b, 1.0f);
        if (out_rgba8) {
            r = fmaxf(r, 0.0f);  // saveImage clamps negative values before the gamma
            g = fmaxf(g, 0.0f);
            b = fmaxf(b, 0.0f);
            if (flags & VPT_SDR_SRGB) {
                r = srgb_gamma(r);
                g = srgb_gamma(g);
                b = srgb_gamma(b);
            }
            const int64_t y = i / width, x = i - y * width;
            const int64_t dst = (flags & VPT_SDR_FLIP_Y) ? (height - 1 - y) * width + x : i;
            out_rgba8[dst] = to_byte(r) | (to_byte(g) << 8) | (to_byte(b) << 16) | (255u << 24);
        }
    }
}

}  // namespace

int launch_tonemap(VptContextImpl* c, cudaStream_t s, float brightness, uint32_t flags, float* rgba32,
                   uint32_t* rgba8) {
    const int64_t n = static_cast<int64_t>(c->width) * c->height;
    const int blocks = static_cast<int>(std::min<int64_t>((n + 255) / 256, static_cast<int64_t>(c->num_sms) * 8));
    tonemap_kernel<<<blocks, 256, 0, s>>>(c->d_mean, c->width, c->height, brightness, flags,
                                          reinterpret_cast<float4*>(rgba32), rgba8);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return ctx_set_error(VPT_ERR_CUDA, cudaGetErrorString(e));
    return VPT_OK;
}

}  // namespace vpt

extern "C" {

int vpt_tonemap(VptContext* c, void* stream, float brightness, uint32_t sdr_flags, float* dev_rgba32,
                uint32_t* dev_rgba8) {
    if (!c || !(brightness >= 0.0f)) return vpt::ctx_set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_tonemap: bad arguments");
    if (!dev_rgba32 && !dev_rgba8) return VPT_OK;
    return vpt::launch_tonemap(c, static_cast<cudaStream_t>(stream), brightness, sdr_flags, dev_rgba32, dev_rgba8);
}

int vpt_download_image_rgba8(VptContext* c, float brightness, uint32_t sdr_flags, uint32_t* host_rgba8) {
    if (!c || !host_rgba8 || !(brightness >= 0.0f))
        return vpt::ctx_set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_download_image_rgba8: bad arguments");
    const size_t n = static_cast<size_t>(c->width) * c->height;
    if (!c->d_rgba8) {
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&c->d_rgba8), n * sizeof(uint32_t));
        if (e != cudaSuccess) {
            c->d_rgba8 = nullptr;
            return vpt::ctx_set_error(VPT_ERR_OUT_OF_MEMORY, cudaGetErrorString(e));
        }
    }
    int rc = vpt::launch_tonemap(c, nullptr, brightness, sdr_flags, nullptr, c->d_rgba8);
    if (rc) return rc;
    const cudaError_t e = cudaMemcpy(host_rgba8, c->d_rgba8, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return vpt::ctx_set_error(VPT_ERR_CUDA, cudaGetErrorString(e));
    return VPT_OK;
}

}  // extern "C"
