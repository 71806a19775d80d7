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
            contribution = max0(load_rgb(b.inferred + 3 * static_cast<size_t>(i)));
            if (radiance_scale > 0) contribution = rdiv(contribution, radiance_scale);
            contribution = contribution * reflectance(b.infer_query + kQueryFloats * static_cast<size_t>(i));
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

// nrc_set_up_kernels.cu:88-174 (one thread per slot of the 2^16-sample training batch).
__global__ void shuffle_kernel(NrcBuffers b, uint32_t buf, float radiance_scale) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNumTrainingDataPerFrame) return;
    const uint32_t num = b.counters[buf];
    if (num > 0) {
        // renderer_shared.h:92-109: state = (state * 1103515245 + 12345) mod 2^31 (u32 arithmetic).
        uint32_t st = b.shufflers[i];
        st = (st * 1103515245u + 12345u) % (1u << 31);
        b.shufflers[i] = st;
        const uint32_t dst = st % kNumTrainingDataPerFrame;
        const uint32_t src = i % num;
        float q[kQueryFloats];
#pragma unroll
        for (int k = 0; k < kQueryFloats; ++k) q[k] = b.train_query[0][kQueryFloats * static_cast<size_t>(src) + k];
        RGB target = load_rgb(b.train_target[0] + 3 * static_cast<size_t>(src));
        if (!all_finite_query(q)) {
#pragma unroll
            for (int k = 0; k < kQueryFloats; ++k) q[k] = 0.0f;
        }
        if (!all_nonneg_finite(target)) target = rgb(0, 0, 0);
        // Batch statistics (targetMinMax / targetAvg): non-negative floats order like their bits.
        float* s = b.stats + 9 * buf;
        atomicMin(reinterpret_cast<unsigned int*>(s + 0), __float_as_uint(target.r));
        atomicMin(reinterpret_cast<unsigned int*>(s + 1), __float_as_uint(target.g));
        atomicMin(reinterpret_cast<unsigned int*>(s + 2), __float_as_uint(target.b));
        atomicMax(reinterpret_cast<int*>(s + 3), __float_as_int(target.r));
        atomicMax(reinterpret_cast<int*>(s + 4), __float_as_int(target.g));
        atomicMax(reinterpret_cast<int*>(s + 5), __float_as_int(target.b));
        atomicAdd(s + 6, target.r / kNumTrainingDataPerFrame);
        atomicAdd(s + 7, target.g / kNumTrainingDataPerFrame);
        atomicAdd(s + 8, target.b / kNumTrainingDataPerFrame);
        if (radiance_scale > 0) target = target * radiance_scale;
        target = rgb(fminf(target.r, 1e6f), fminf(target.g, 1e6f), fminf(target.b, 1e6f));
#pragma unroll
        for (int k = 0; k < kQueryFloats; ++k) b.train_query[1][kQueryFloats * static_cast<size_t>(dst) + k] = q[k];
        store_rgb(b.train_target[1] + 3 * static_cast<size_t>(dst), target);
    } else {
#pragma unroll
        for (int k = 0; k < kQueryFloats; ++k) b.train_query[1][kQueryFloats * static_cast<size_t>(i) + k] = 0.0f;
        store_rgb(b.train_target[1] + 3 * static_cast<size_t>(i), rgb(0, 0, 0));
    }
}

// nrc_set_up_kernels.cu:176-219, accumulating into both the reference's FP32 running mean and
// the FP64 sums.
__global__ void accumulate_kernel(NrcBuffers b, float radiance_scale, uint32_t accum_frames, double* __restrict__ sum,
                                  float* __restrict__ mean, unsigned int* __restrict__ err) {
    const uint32_t npix = static_cast<uint32_t>(b.width) * static_cast<uint32_t>(b.height);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
        const TerminalInfo t = b.infer_terminal[i];
        RGB direct = load_rgb(b.frame_contribution + 3 * static_cast<size_t>(i));
        RGB radiance = rgb(0, 0, 0);
        if (t.bits & 1u) {
            radiance = max0(load_rgb(b.inferred + 3 * static_cast<size_t>(i)));
            if (radiance_scale > 0) radiance = rdiv(radiance, radiance_scale);
            radiance = radiance * reflectance(b.infer_query + kQueryFloats * static_cast<size_t>(i));
        }
        RGB c = direct + rgb(t.tp[0], t.tp[1], t.tp[2]) * radiance;
        if (!all_nonneg_finite(c)) {
            atomicOr(err, 2u);
            c = rgb(0, 0, 0);
        }
        RGB prev = accum_frames > 0 ? load_rgb(mean + 3 * static_cast<size_t>(i)) : rgb(0, 0, 0);
        float w = 1.0f / (accum_frames + 1);
        store_rgb(mean + 3 * static_cast<size_t>(i), (1 - w) * prev + w * c);
        sum[3 * static_cast<size_t>(i)] += c.r;
        sum[3 * static_cast<size_t>(i) + 1] += c.g;
        sum[3 * static_cast<size_t>(i) + 2] += c.b;
    }
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
    shuffle_kernel<<<kNumTrainingDataPerFrame / 256, 256, 0, s>>>(b, buf, radiance_scale);
}
void nrc_accumulate(const NrcBuffers& b, float radiance_scale, uint32_t accum_frames, double* sum, float* mean,
                    unsigned int* err, cudaStream_t s) {
    uint32_t n = static_cast<uint32_t>(b.width) * static_cast<uint32_t>(b.height);
    accumulate_kernel<<<(n + 255) / 256, 256, 0, s>>>(b, radiance_scale, accum_frames, sum, mean, err);
}

}  // namespace vpt
