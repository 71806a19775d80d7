/*
 * ORACLE (test infrastructure only) — CPU restatement of the radiance-cache set-up kernels
 * between the tracer passes (renderer/gpu_kernels/nrc_set_up_kernels.cu) and of the shuffler
 * initialisation (renderer/renderer_main.cpp:218-229), on host arrays in the device layouts.
 *
 * Parity status: pinned to the reference's source text of these kernels (they are plain
 * arithmetic on the buffers; no reference build is needed to restate them). Suffix walks
 * and shuffles run sequentially here; the device runs them in parallel, where only the
 * write order of colliding shuffle slots and the summation order of the batch average
 * differ (the tests compare slots with one writer and the average within a tolerance).
 */
#include <cmath>
#include <cstdint>
#include <cstring>

#include "vpt_oracle.h"

namespace {

constexpr uint32_t kTrainPerFrame = 65536u;  // numTrainingDataPerFrame (renderer_shared.h:12)

inline float max0(float x) { return x > 0.0f ? x : 0.0f; }  // max(x, 0) of RGBSpectrum
inline float safe_div(float a, float b) { return b != 0.0f ? a / b : 0.0f; }  // basic_types.h:3094-3102
inline bool finite_nonneg(const float* c) {
    return std::isfinite(c[0]) && std::isfinite(c[1]) && std::isfinite(c[2]) && c[0] >= 0 && c[1] >= 0 && c[2] >= 0;
}
inline uint32_t lcg_next(uint32_t s) { return (s * 1103515245u + 12345u) % (1u << 31); }  // renderer_shared.h:92-109

// Cache prediction at a terminal query: max(NN, 0) / radianceScale * (diffuse + specular).
inline void terminal_radiance(const float* inferred, const float* q, float radiance_scale, float* out) {
    for (int c = 0; c < 3; ++c) {
        float v = max0(inferred[c]);
        if (radiance_scale > 0) v = v / radiance_scale;
        out[c] = v * (q[8 + c] + q[11 + c]);
    }
}

}  // namespace

extern "C" {

// renderer_main.cpp:218-229: shuffler i = LCG state after i + 1 steps from 471313181.
void orc_nrc_shufflers(uint32_t* out) {
    uint32_t s = 471313181u;
    for (uint32_t i = 0; i < kTrainPerFrame; ++i) {
        s = lcg_next(s);
        out[i] = s;
    }
}

// nrc_set_up_kernels.cu:4-44.
void orc_nrc_prepare(uint32_t* counters, float* stats, uint32_t* train_suffix, int32_t width, int32_t height,
                     uint32_t buf, uint32_t offset, int32_t new_sequence) {
    const uint32_t prev = (buf + 1) % 2;
    int nx, ny;
    if (new_sequence) {
        nx = width / 4;
        ny = height / 4;
    } else {
        float r = std::sqrt(static_cast<float>(counters[prev]) / kTrainPerFrame);
        int cx = static_cast<int>(counters[2 + 2 * prev]), cy = static_cast<int>(counters[3 + 2 * prev]);
        nx = static_cast<int>(std::fmin(cx / r, static_cast<float>(width)));
        ny = static_cast<int>(std::fmin(cy / r, static_cast<float>(height)));
    }
    counters[2 + 2 * buf] = static_cast<uint32_t>(nx);
    counters[3 + 2 * buf] = static_cast<uint32_t>(ny);
    counters[buf] = 0;
    counters[6] = offset;
    counters[7] = static_cast<uint32_t>(nx) * static_cast<uint32_t>(ny);
    float* s = stats + 9 * buf;
    for (int c = 0; c < 3; ++c) {
        s[c] = INFINITY;
        s[3 + c] = -INFINITY;
        s[6 + c] = 0.0f;
    }
    const uint32_t n = static_cast<uint32_t>(width) * static_cast<uint32_t>(height);
    for (uint32_t i = 0; i < n; ++i) train_suffix[i] = ORC_NRC_INVALID_VERTEX;  // prev invalid, no query, length 0
}

// nrc_set_up_kernels.cu:46-86. vertex: 4 words per vertex (local throughput rgb, bits).
void orc_nrc_propagate(uint32_t num_suffixes, const uint32_t* train_suffix, const float* inferred,
                       const float* infer_query, const float* vertex, const float* train_query0, float* train_target0,
                       float radiance_scale) {
    for (uint32_t i = 0; i < num_suffixes; ++i) {
        const uint32_t term = train_suffix[i];
        uint32_t idx = term & ORC_NRC_INVALID_VERTEX;
        if (idx >= ORC_NRC_TRAIN_BUFFER_SIZE) continue;
        float contribution[3] = {0, 0, 0};
        if ((term >> 22) & 1u)
            terminal_radiance(inferred + 3 * static_cast<size_t>(i), infer_query + 14 * static_cast<size_t>(i),
                              radiance_scale, contribution);
        for (uint32_t guard = 0; idx < ORC_NRC_TRAIN_BUFFER_SIZE && guard < ORC_NRC_TRAIN_BUFFER_SIZE; ++guard) {
            const float* v = vertex + 4 * static_cast<size_t>(idx);
            float* target = train_target0 + 3 * static_cast<size_t>(idx);
            const float* q = train_query0 + 14 * static_cast<size_t>(idx);
            for (int c = 0; c < 3; ++c) {
                float indirect = v[c] * contribution[c];
                contribution[c] = target[c] + indirect;
                target[c] = safe_div(contribution[c], q[8 + c] + q[11 + c]);
            }
            uint32_t bits;
            std::memcpy(&bits, v + 3, 4);
            idx = bits & ORC_NRC_INVALID_VERTEX;
        }
    }
}

// nrc_set_up_kernels.cu:88-174, threads in index order. writers[dst] (may be null) counts the
// threads that wrote slot dst of buffer 1.
void orc_nrc_shuffle(uint32_t num_training, float* stats_buf, uint32_t* shufflers, const float* train_query0,
                     const float* train_target0, float* train_query1, float* train_target1, float radiance_scale,
                     uint32_t* writers) {
    double avg[3] = {0, 0, 0};
    for (uint32_t i = 0; i < kTrainPerFrame; ++i) {
        if (num_training == 0) {
            std::memset(train_query1 + 14 * static_cast<size_t>(i), 0, 14 * sizeof(float));
            std::memset(train_target1 + 3 * static_cast<size_t>(i), 0, 3 * sizeof(float));
            if (writers) ++writers[i];
            continue;
        }
        shufflers[i] = lcg_next(shufflers[i]);
        const uint32_t dst = shufflers[i] % kTrainPerFrame;
        const uint32_t src = i % num_training;
        float q[14], t[3];
        std::memcpy(q, train_query0 + 14 * static_cast<size_t>(src), sizeof(q));
        std::memcpy(t, train_target0 + 3 * static_cast<size_t>(src), sizeof(t));
        bool valid = true;
        for (int k = 0; k < 14; ++k) valid = valid && std::isfinite(q[k]);
        if (!valid) std::memset(q, 0, sizeof(q));
        if (!finite_nonneg(t)) t[0] = t[1] = t[2] = 0.0f;
        for (int c = 0; c < 3; ++c) {
            stats_buf[c] = std::fmin(stats_buf[c], t[c]);
            stats_buf[3 + c] = std::fmax(stats_buf[3 + c], t[c]);
            avg[c] += static_cast<double>(t[c] / kTrainPerFrame);
        }
        for (int c = 0; c < 3; ++c) {
            if (radiance_scale > 0) t[c] = t[c] * radiance_scale;
            t[c] = std::fmin(t[c], 1e6f);
        }
        std::memcpy(train_query1 + 14 * static_cast<size_t>(dst), q, sizeof(q));
        std::memcpy(train_target1 + 3 * static_cast<size_t>(dst), t, sizeof(t));
        if (writers) ++writers[dst];
    }
    if (num_training > 0)
        for (int c = 0; c < 3; ++c) stats_buf[6 + c] += static_cast<float>(avg[c]);
}

// nrc_set_up_kernels.cu:176-219 (FP32 running mean as sample `accum_frames`) and the FP64 sums.
// terminal: 4 words per pixel (throughput rgb, bits). Non-finite results count as 0.
void orc_nrc_accumulate(uint32_t num_pixels, const float* terminal, const float* frame_contribution,
                        const float* inferred, const float* infer_query, float radiance_scale, uint32_t accum_frames,
                        double* sum, float* mean) {
    for (uint32_t i = 0; i < num_pixels; ++i) {
        const float* t = terminal + 4 * static_cast<size_t>(i);
        uint32_t bits;
        std::memcpy(&bits, t + 3, 4);
        float radiance[3] = {0, 0, 0};
        if (bits & 1u)
            terminal_radiance(inferred + 3 * static_cast<size_t>(i), infer_query + 14 * static_cast<size_t>(i),
                              radiance_scale, radiance);
        float c[3];
        for (int k = 0; k < 3; ++k) c[k] = frame_contribution[3 * static_cast<size_t>(i) + k] + t[k] * radiance[k];
        if (!finite_nonneg(c)) c[0] = c[1] = c[2] = 0.0f;
        const float w = 1.0f / (accum_frames + 1);
        for (int k = 0; k < 3; ++k) {
            float prev = accum_frames > 0 ? mean[3 * static_cast<size_t>(i) + k] : 0.0f;
            mean[3 * static_cast<size_t>(i) + k] = (1 - w) * prev + w * c[k];
            sum[3 * static_cast<size_t>(i) + k] += c[k];
        }
    }
}

}  // extern "C"
