// Radiance-cache set-up kernels (renderer/gpu_kernels/nrc_set_up_kernels.cu:4-219): the
// adaptive training-image size, back-propagation of cache predictions along the training
// suffixes, the LCG shuffle into the training batch, and the final per-pixel accumulation.
// The training-image size and query counts stay on the device (the reference reads the size
// back to the host with a stream synchronisation, renderer/renderer_main.cpp:1568-1573).
#include <cuda_runtime.h>

#include "nrc_buffers.cuh"
#include "vpt_device.cuh"

namespace vpt {
namespace {

__device__ __forceinline__ RGB load_rgb(const float* p) { return rgb(p[0], p[1], p[2]); }
__device__ __forceinline__ void store_rgb(float* p, RGB c) {
    p[0] = c.r;
    p[1] = c.g;
    p[2] = c.b;
}
__device__ __forceinline__ RGB max0(RGB c) { return rgb(fmaxf(c.r, 0.0f), fmaxf(c.g, 0.0f), fmaxf(c.b, 0.0f)); }
// basic_types.h:3094-3102 (component-wise a / b, 0 where b == 0).
__device__ __forceinline__ RGB safe_divide(RGB a, RGB b) {
    return rgb(b.r != 0 ? a.r / b.r : 0.0f, b.g != 0 ? a.g / b.g : 0.0f, b.b != 0 ? a.b / b.b : 0.0f);
}
__device__ __forceinline__ RGB reflectance(const float* q) {  // diffuse + specular of a RadianceQuery
    return rgb(q[8] + q[11], q[9] + q[12], q[10] + q[13]);
}

// nrc_set_up_kernels.cu:4-44.
__global__ void prepare_kernel(NrcBuffers b, uint32_t buf, uint32_t offset, int new_sequence) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.max_train_suffixes) return;
    if (i == 0) {
        uint32_t prev = (buf + 1) % 2;
        int nx, ny;
        if (new_sequence) {
            nx = b.width / 4;
            ny = b.height / 4;
        } else {
            uint32_t prev_num = b.counters[prev];
            float r = sqrtf(static_cast<float>(prev_num) / kNumTrainingDataPerFrame);
            int cx = static_cast<int>(b.counters[2 + 2 * prev]), cy = static_cast<int>(b.counters[3 + 2 * prev]);
            nx = static_cast<int>(fminf(cx / r, static_cast<float>(b.width)));
            ny = static_cast<int>(fminf(cy / r, static_cast<float>(b.height)));
        }
        b.counters[2 + 2 * buf] = static_cast<uint32_t>(nx);
        b.counters[3 + 2 * buf] = static_cast<uint32_t>(ny);
        b.counters[buf] = 0;
        b.counters[6] = offset;
        b.counters[7] = static_cast<uint32_t>(nx) * static_cast<uint32_t>(ny);
        float* s = b.stats + 9 * buf;
        for (int c = 0; c < 3; ++c) {
            s[c] = INFINITY;
            s[3 + c] = -INFINITY;
            s[6 + c] = 0.0f;
        }
    }
    b.train_suffix[i] = pack_suffix(kInvalidVertex, 0, 0, 0);
}

// nrc_set_up_kernels.cu:46-86.
__global__ void propagate_kernel(NrcBuffers b, float radiance_scale) {
    const uint32_t n = b.counters[7];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n && i < b.max_train_suffixes;
         i += gridDim.x * blockDim.x) {
        uint32_t term = b.train_suffix[i];
        uint32_t idx = term & kInvalidVertex;
        if (idx >= kTrainBufferSize) continue;  // no vertex (kInvalidVertex) or a corrupt link
        RGB contribution = rgb(0, 0, 0);
        if ((term >> 22) & 1u) {
            contribution = max0(load_rgb(b.train_end_inferred + 3 * static_cast<size_t>(i)));
            if (radiance_scale > 0) contribution = rdiv(contribution, radiance_scale);
            contribution = contribution * reflectance(b.train_end_query + kQueryFloats * static_cast<size_t>(i));
        }
        // Walk the suffix backwards; vertex indices decrease along it, so the walk ends.
        for (uint32_t guard = 0; idx < kTrainBufferSize && guard < kTrainBufferSize; ++guard) {
            const TrainVertexInfo vi = b.train_vertex[idx];
            float* target = b.train_target[0] + 3 * static_cast<size_t>(idx);
            RGB indirect = rgb(vi.local_tp[0], vi.local_tp[1], vi.local_tp[2]) * contribution;
            contribution = load_rgb(target) + indirect;
            store_rgb(target, safe_divide(contribution, reflectance(b.train_query[0] + kQueryFloats * static_cast<size_t>(idx))));
            idx = vi.bits & kInvalidVertex;
        }
    }
}

__device__ __forceinline__ bool all_finite_query(const float* q) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < kQueryFloats; ++k) ok = ok && isfinite(q[k]);
    return ok;
}

// nrc_set_up_kernels.cu:88-174 (one thread per slot of the 2^16-sample training batch). The batch
// statistics are reduced per block first (warp shuffles, then shared memory), so each block
// issues one atomic per statistic, as the reference's block-level atomics do (:132-150).
constexpr int kShuffleThreads = 256;
__global__ void __launch_bounds__(kShuffleThreads) shuffle_kernel(NrcBuffers b, uint32_t buf, float radiance_scale) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < kNumTrainingDataPerFrame;
    const uint32_t num = b.counters[buf];  // uniform over the grid
    if (num == 0) {
        if (!active) return;
#pragma unroll
        for (int k = 0; k < kQueryFloats; ++k) b.train_query[1][kQueryFloats * static_cast<size_t>(i) + k] = 0.0f;
        store_rgb(b.train_target[1] + 3 * static_cast<size_t>(i), rgb(0, 0, 0));
        return;
    }
    // Neutral values for threads beyond the batch (none with the exact grid used below).
    RGB target = rgb(0, 0, 0);
    RGB tmin = rgb(INFINITY, INFINITY, INFINITY), tmax = rgb(-INFINITY, -INFINITY, -INFINITY);
    RGB tavg = rgb(0, 0, 0);
    uint32_t dst = 0;
    float q[kQueryFloats];
    if (active) {
        // renderer_shared.h:92-109: state = (state * 1103515245 + 12345) mod 2^31 (u32 arithmetic).
        uint32_t st = b.shufflers[i];
        st = (st * 1103515245u + 12345u) % (1u << 31);
        b.shufflers[i] = st;
        dst = st % kNumTrainingDataPerFrame;
        const uint32_t src = i % num;
#pragma unroll
        for (int k = 0; k < kQueryFloats; ++k) q[k] = b.train_query[0][kQueryFloats * static_cast<size_t>(src) + k];
        target = load_rgb(b.train_target[0] + 3 * static_cast<size_t>(src));
        if (!all_finite_query(q)) {
#pragma unroll
            for (int k = 0; k < kQueryFloats; ++k) q[k] = 0.0f;
        }
        if (!all_nonneg_finite(target)) target = rgb(0, 0, 0);
        tmin = tmax = target;
        tavg = rdiv(target, static_cast<float>(kNumTrainingDataPerFrame));
    }
    // Batch statistics (targetMinMax / targetAvg).
    float v[9] = {tmin.r, tmin.g, tmin.b, tmax.r, tmax.g, tmax.b, tavg.r, tavg.g, tavg.b};
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[c] = fminf(v[c], __shfl_xor_sync(0xffffffffu, v[c], off));
            v[3 + c] = fmaxf(v[3 + c], __shfl_xor_sync(0xffffffffu, v[3 + c], off));
            v[6 + c] += __shfl_xor_sync(0xffffffffu, v[6 + c], off);
        }
    }
    __shared__ float s_red[kShuffleThreads / 32][9];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 9; ++k) s_red[warp][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        const int k = threadIdx.x;
        float r = s_red[0][k];
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) {
            const float x = s_red[w][k];
            r = k < 3 ? fminf(r, x) : (k < 6 ? fmaxf(r, x) : r + x);
        }
        float* s = b.stats + 9 * buf;
        // Non-negative floats order like their bit patterns (min starts at +inf, max at -inf).
        if (k < 3)
            atomicMin(reinterpret_cast<unsigned int*>(s + k), __float_as_uint(r));
        else if (k < 6)
            atomicMax(reinterpret_cast<int*>(s + k), __float_as_int(r));
        else
            atomicAdd(s + k, r);
    }
    if (!active) return;
    if (radiance_scale > 0) target = target * radiance_scale;
    target = rgb(fminf(target.r, 1e6f), fminf(target.g, 1e6f), fminf(target.b, 1e6f));
#pragma unroll
    for (int k = 0; k < kQueryFloats; ++k) b.train_query[1][kQueryFloats * static_cast<size_t>(dst) + k] = q[k];
    store_rgb(b.train_target[1] + 3 * static_cast<size_t>(dst), target);
}

// nrc_set_up_kernels.cu:176-219 for `spp` samples per pixel (slot = sample * pixels + pixel),
// added to the FP64 sums. spp == 1 without `from_sums` keeps the reference's FP32 running mean
// as sample `accum_frames`; otherwise the mean is the FP64 sum over accum_frames + spp samples.
__global__ void accumulate_kernel(NrcBuffers b, float radiance_scale, uint32_t accum_frames, uint32_t spp,
                                  int from_sums, double* __restrict__ sum, float* __restrict__ mean,
                                  unsigned int* __restrict__ err) {
    const uint32_t npix = static_cast<uint32_t>(b.width) * static_cast<uint32_t>(b.height);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
        double acc[3] = {0, 0, 0};
        RGB c = rgb(0, 0, 0);
        for (uint32_t smp = 0; smp < spp; ++smp) {
            const size_t slot = static_cast<size_t>(smp) * npix + i;
            const TerminalInfo t = b.infer_terminal[slot];
            RGB direct = load_rgb(b.frame_contribution + 3 * slot);
            RGB radiance = rgb(0, 0, 0);
            if (t.bits & 1u) {
                radiance = max0(load_rgb(b.inferred + 3 * slot));
                if (radiance_scale > 0) radiance = rdiv(radiance, radiance_scale);
                radiance = radiance * reflectance(b.infer_query + kQueryFloats * slot);
            }
            c = direct + rgb(t.tp[0], t.tp[1], t.tp[2]) * radiance;
            if (!all_nonneg_finite(c)) {
                atomicOr(err, 2u);
                c = rgb(0, 0, 0);
            }
            acc[0] += c.r;
            acc[1] += c.g;
            acc[2] += c.b;
        }
        const double s0 = sum[3 * static_cast<size_t>(i)] + acc[0];
        const double s1 = sum[3 * static_cast<size_t>(i) + 1] + acc[1];
        const double s2 = sum[3 * static_cast<size_t>(i) + 2] + acc[2];
        sum[3 * static_cast<size_t>(i)] = s0;
        sum[3 * static_cast<size_t>(i) + 1] = s1;
        sum[3 * static_cast<size_t>(i) + 2] = s2;
        if (spp == 1 && !from_sums) {
            RGB prev = accum_frames > 0 ? load_rgb(mean + 3 * static_cast<size_t>(i)) : rgb(0, 0, 0);
            float w = 1.0f / (accum_frames + 1);
            store_rgb(mean + 3 * static_cast<size_t>(i), (1 - w) * prev + w * c);
        } else {
            const double inv = 1.0 / (static_cast<double>(accum_frames) + spp);
            store_rgb(mean + 3 * static_cast<size_t>(i), rgb(static_cast<float>(s0 * inv), static_cast<float>(s1 * inv),
                                                               static_cast<float>(s2 * inv)));
        }
    }
}

// accumulate_kernel for spp > 1 with the samples spread over the threads: a block covers 32
// pixels, its 8 warps take every 8th sample of them (coalesced loads of consecutive pixels'
// slots), and the partial sums are added in shared memory in warp order.
constexpr int kAccumParts = 8;
__global__ void __launch_bounds__(32 * kAccumParts) accumulate_parallel_kernel(NrcBuffers b, float radiance_scale,
                                                                               uint32_t accum_frames, uint32_t spp,
                                                                               double* __restrict__ sum,
                                                                               float* __restrict__ mean,
                                                                               unsigned int* __restrict__ err) {
    __shared__ double s_acc[kAccumParts][32][3];
    const uint32_t npix = static_cast<uint32_t>(b.width) * static_cast<uint32_t>(b.height);
    const uint32_t lane = threadIdx.x & 31, part = threadIdx.x >> 5;
    const uint32_t i = blockIdx.x * 32 + lane;
    double acc[3] = {0, 0, 0};
    if (i < npix) {
        for (uint32_t smp = part; smp < spp; smp += kAccumParts) {
            const size_t slot = static_cast<size_t>(smp) * npix + i;
            const TerminalInfo t = b.infer_terminal[slot];
            const RGB direct = load_rgb(b.frame_contribution + 3 * slot);
            RGB radiance = rgb(0, 0, 0);
            if (t.bits & 1u) {
                radiance = max0(load_rgb(b.inferred + 3 * slot));
                if (radiance_scale > 0) radiance = rdiv(radiance, radiance_scale);
                radiance = radiance * reflectance(b.infer_query + kQueryFloats * slot);
            }
            RGB c = direct + rgb(t.tp[0], t.tp[1], t.tp[2]) * radiance;
            if (!all_nonneg_finite(c)) {
                atomicOr(err, 2u);
                c = rgb(0, 0, 0);
            }
            acc[0] += c.r;
            acc[1] += c.g;
            acc[2] += c.b;
        }
    }
    s_acc[part][lane][0] = acc[0];
    s_acc[part][lane][1] = acc[1];
    s_acc[part][lane][2] = acc[2];
    __syncthreads();
    if (part != 0 || i >= npix) return;
    double t0 = 0, t1 = 0, t2 = 0;
#pragma unroll
    for (int w = 0; w < kAccumParts; ++w) {
        t0 += s_acc[w][lane][0];
        t1 += s_acc[w][lane][1];
        t2 += s_acc[w][lane][2];
    }
    const double s0 = sum[3 * static_cast<size_t>(i)] + t0;
    const double s1 = sum[3 * static_cast<size_t>(i) + 1] + t1;
    const double s2 = sum[3 * static_cast<size_t>(i) + 2] + t2;
    sum[3 * static_cast<size_t>(i)] = s0;
    sum[3 * static_cast<size_t>(i) + 1] = s1;
    sum[3 * static_cast<size_t>(i) + 2] = s2;
    const double inv = 1.0 / (static_cast<double>(accum_frames) + spp);
    store_rgb(mean + 3 * static_cast<size_t>(i),
              rgb(static_cast<float>(s0 * inv), static_cast<float>(s1 * inv), static_cast<float>(s2 * inv)));
}

}  // namespace

void nrc_prepare(const NrcBuffers& b, uint32_t buf, uint32_t offset, bool new_sequence, cudaStream_t s) {
    uint32_t n = b.max_train_suffixes;
    prepare_kernel<<<(n + 255) / 256, 256, 0, s>>>(b, buf, offset, new_sequence ? 1 : 0);
}
void nrc_propagate(const NrcBuffers& b, float radiance_scale, cudaStream_t s) {
    uint32_t n = b.max_train_suffixes;
    propagate_kernel<<<(n + 255) / 256, 256, 0, s>>>(b, radiance_scale);
}
void nrc_shuffle(const NrcBuffers& b, uint32_t buf, float radiance_scale, cudaStream_t s) {
    shuffle_kernel<<<kNumTrainingDataPerFrame / kShuffleThreads, kShuffleThreads, 0, s>>>(b, buf, radiance_scale);
}
void nrc_accumulate(const NrcBuffers& b, float radiance_scale, uint32_t accum_frames, uint32_t spp, bool from_sums,
                    double* sum, float* mean, unsigned int* err, cudaStream_t s) {
    uint32_t n = static_cast<uint32_t>(b.width) * static_cast<uint32_t>(b.height);
    if (spp > 1) {
        accumulate_parallel_kernel<<<(n + 31) / 32, 32 * kAccumParts, 0, s>>>(b, radiance_scale, accum_frames, spp, sum,
                                                                              mean, err);
        return;
    }
    accumulate_kernel<<<(n + 255) / 256, 256, 0, s>>>(b, radiance_scale, accum_frames, spp, from_sums ? 1 : 0, sum, mean,
                                                      err);
}

}  // namespace vpt
