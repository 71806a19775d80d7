// Device buffers of the radiance-cache render / training passes (the reference's NRC buffers,
// renderer/renderer_main.cpp:60-79, 197-230, and their fields in StaticPipelineLaunchParameters,
// renderer/renderer_shared.h:127-141).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace vpt {

constexpr uint32_t kNumTrainingDataPerFrame = 1u << 16;               // renderer_shared.h:12
constexpr uint32_t kTrainBufferSize = 2 * kNumTrainingDataPerFrame;    // renderer_shared.h:13
constexpr float kPathTerminationFactor = 0.01f;                        // renderer_shared.h:11
constexpr uint32_t kInvalidVertex = 0x003FFFFFu;                       // renderer_shared.h:74
constexpr int kQueryFloats = 14;                                       // RadianceQuery, renderer_shared.h:46-54

// TerminalInfo (renderer_shared.h:67-72): throughput + (hasQuery | pathLength << 1).
struct TerminalInfo {
    float tp[3];
    uint32_t bits;
};
// TrainingVertexInfo (renderer_shared.h:76-82): local throughput + (prev | pathLength << 22 | unbiased << 30).
struct TrainVertexInfo {
    float local_tp[3];
    uint32_t bits;
};
// TrainingSuffixTerminalInfo (renderer_shared.h:84-90): prev | hasQuery << 22 | pathLength << 23 | unbiased << 31.
__host__ __device__ __forceinline__ uint32_t pack_suffix(uint32_t prev, uint32_t has_query, uint32_t path_length,
                                                         uint32_t unbiased) {
    return (prev & kInvalidVertex) | ((has_query & 1u) << 22) | ((path_length & 0xFFu) << 23) | ((unbiased & 1u) << 31);
}

// The arrays one training pass writes: several passes traced in one launch (the frame's
// training iterations, vpt_nrc_frame) each get their own set; the shuffled batch, the shufflers
// and the statistics are shared because the sets are post-processed one after the other.
constexpr uint32_t kMaxTrainSets = 4;
struct TrainSet {
    uint32_t* counters;          // as NrcBuffers::counters
    uint64_t* rng;               // per-pixel PCG32 states of the set's training paths
    TrainVertexInfo* vertex;     // kTrainBufferSize
    float* query0;               // kTrainBufferSize * 14 (train_query[0])
    float* target0;              // kTrainBufferSize * 3 (train_target[0])
    float* end_query;            // max_train_suffixes * 14
    float* end_inferred;         // max_train_suffixes * 3
    uint32_t* suffix;            // max_train_suffixes
};

// Device pointers and sizes used by the NRC kernels.
struct NrcBuffers {
    int32_t width = 0, height = 0;   // render image
    uint32_t max_train_suffixes = 0; // = width * height (renderer_main.cpp:113)
    uint32_t infer_capacity = 0;     // roundUp(width * height * render_spp, 128)
    uint32_t render_spp = 1;         // sample slots per pixel of the render-pass buffers

    float* infer_query = nullptr;        // infer_capacity * 14
    TerminalInfo* infer_terminal = nullptr;  // width * height * render_spp
    uint32_t* train_suffix = nullptr;    // max_train_suffixes
    float* inferred = nullptr;           // infer_capacity * 3
    float* frame_contribution = nullptr; // width * height * render_spp * 3
    // Slots of the render queries a pass wrote (count in counters[8]), so that inference runs on
    // those records only; null = the pass does not list them (inference over every slot, as the
    // reference does).
    uint32_t* infer_index = nullptr;     // width * height * render_spp
    float* train_query[2] = {nullptr, nullptr};   // kTrainBufferSize * 14
    float* train_target[2] = {nullptr, nullptr};  // kTrainBufferSize * 3
    TrainVertexInfo* train_vertex = nullptr;      // kTrainBufferSize
    // End queries of the training suffixes and their predictions (max_train_suffixes records).
    // The reference keeps them in the render pass's inference buffers and serialises the passes
    // (renderer_main.cpp:1611-1613); separate buffers let the two passes run concurrently.
    float* train_end_query = nullptr;             // max_train_suffixes * 14
    float* train_end_inferred = nullptr;          // max_train_suffixes * 3
    // Per-pixel PCG32 states of the training pass when the render passes use sample-parallel
    // streams (the context's states, advanced 2^62 draws); null = the context's states.
    uint64_t* train_rng = nullptr;
    uint32_t* shufflers = nullptr;                // kNumTrainingDataPerFrame LCG states
    // [0..1] numTrainingData per buffer, [2..5] trainImageSize (x, y) per buffer,
    // [6] offsetToSelectUnbiasedPath, [7] training-pass query count of the current buffer
    // (trainW * trainH), [8] render queries listed in infer_index, [9..15] unused.
    uint32_t* counters = nullptr;
    float* stats = nullptr;          // per buffer: min rgb, max rgb, avg rgb (9 floats)
    uint32_t buffer_index = 0;       // nrcBufferIndex of the current training iteration
    // Training sets of a multi-pass launch: set 0 is the arrays above, sets 1.. are allocated on
    // first use; `train_sets` is the device table of all of them.
    TrainSet sets[kMaxTrainSets] = {};
    uint32_t num_sets = 0;           // sets allocated (0 until the first multi-pass frame)
    TrainSet* train_sets = nullptr;  // device copy of sets[0 .. num_sets)
    uint32_t set_buf[kMaxTrainSets] = {1, 1, 1, 1};  // nrcBufferIndex of each set's last pass
};

// Set-up kernels between the passes (nrc_setup.cu).
void nrc_prepare(const NrcBuffers& b, uint32_t buf, uint32_t offset, bool new_sequence, cudaStream_t s);
void nrc_propagate(const NrcBuffers& b, float radiance_scale, cudaStream_t s);
void nrc_shuffle(const NrcBuffers& b, uint32_t buf, float radiance_scale, cudaStream_t s);
void nrc_accumulate(const NrcBuffers& b, float radiance_scale, uint32_t accum_frames, uint32_t spp, bool from_sums,
                    double* sum, float* mean, unsigned int* err, cudaStream_t s);

}  // namespace vpt
