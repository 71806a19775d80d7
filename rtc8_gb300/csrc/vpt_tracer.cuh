// Launch parameters and kernel declarations of the persistent volumetric tracker.
#pragma once

#include "nrc_buffers.cuh"
#include "vpt_device.cuh"
#include "vpt_surface.cuh"
#include "../../include/rtc8_vpt.h"

namespace vpt {

// Tracer passes (the reference's ray-generation programs).
constexpr int kModePlain = 0;      // pathTrace: accumulate full paths
constexpr int kModeRenderNrc = 1;  // pathTraceWithNRC: short paths ending in a cache query
constexpr int kModeTrainNrc = 2;   // generateTrainingData: training suffixes on the training image
constexpr int kModeComboNrc = 3;   // a training pass and a batched render pass in one launch

struct Sun {
    float dir[3];
    float irradiance[3];
    float select_prob;
    int32_t enabled;
};

// One launch of the tracker. Plain kernel parameter (lives in the constant bank).
struct TraceParams {
    Grid grid;
    Env env;
    Sun sun;
    int32_t env_enabled;

    float cam_aspect, cam_fovy;
    float cam_pos[3];
    float cam_quat[4];
    int32_t width, height;

    float density_coeff, albedo;
    int32_t phase_kind;
    float phase_param;
    float world_radius;
    float world_min[3], world_max[3];  // the world box (volume and instances); the queries' frame

    int32_t max_bounces, rr_start, max_steps;

    uint32_t spp;             // samples per pixel in this launch
    uint32_t accum_base;      // samples already accumulated (numAccumFrames of the first one)
    int32_t stream_mode;      // 0 = per-pixel sequential streams, 1 = sample-parallel streams
    uint32_t stream_base;     // sample-parallel mode: index of the first sample of this launch
    const ulonglong2* sample_jumps;  // sample-parallel mode: LCG jump (A, C) of sample stream_base + i
    int32_t maj_in_smem;      // majorant grid staged in dynamic shared memory
    int32_t park_threshold;   // parked lanes that trigger a warp's event phase (0 = default)
    int32_t leaf_stage_min;   // > 0: per-warp leaf staging when this many lanes look up in one leaf

    uint64_t* rng;            // per pixel
    double* sum_rgb;          // 3 per pixel
    float* mean_rgb;          // 3 per pixel
    uint32_t* dlog;           // optional, 4 per pixel-sample
    unsigned int* work_counter;
    unsigned long long* counters;  // lookups, vertices, samples
    unsigned int* error_flags;

    // Surface scenes only (plain_trace_kernel<..., kSurfaces = true>).
    Surfaces surf;
    int32_t volume_enabled;   // 0: surfaces without a density grid (no tracking, no draws)

    // Radiance-cache passes only.
    NrcBuffers nrc;
    uint32_t nrc_buf;           // training buffer of this frame (nrcBufferIndex)
    // kModeComboNrc: the launch traces num_train_sets training images, set k from the arrays of
    // train_sets[k] with buffer index (train_bufs >> k) & 1, before the render samples.
    const TrainSet* train_sets;
    uint32_t num_train_sets;
    uint32_t train_bufs;
    int32_t nrc_density_query;  // 1: the query's roughness slot carries density / density_coeff
    float nrc_termination;      // path-spread termination factor c (0 = 0.01, renderer_shared.h:11)
    float nrc_train_termination;  // factor of biased training suffixes (0 = 2c)
    float shadow_rr;              // Russian-roulette threshold of shadow-ray visibility (0 = off)
};

// Majorant grids up to this many cells are staged in shared memory (32 KB).
constexpr int kMajSmemCells = 8192;

void launch_plain(const TraceParams& p, bool grid_majorant, int grid_ctas, int threads, size_t smem, cudaStream_t s);
// Dynamic shared memory of a plain launch: the staged majorant grid (`maj_bytes`, 0 if not
// staged) and, with leaf staging, one 2 KB leaf buffer and one mbarrier per warp.
size_t plain_smem_bytes(size_t maj_bytes, bool leaf_stage, int threads);
const void* plain_kernel_ptr(bool grid_majorant, bool logged, bool sample_parallel, bool leaf_stage);
// Plain tracer of scenes with surfaces (either stream layout, logged or not).
const void* surface_kernel_ptr(bool grid_majorant, bool logged);
void launch_surface(const TraceParams& p, bool grid_majorant, int grid_ctas, int threads, size_t smem, cudaStream_t s);
// Threads per CTA of the plain tracer on sample-parallel streams and of the radiance-cache
// passes without meshes (one CTA per SM); the other forms of the tracer run CTAs of 128 threads.
constexpr int kPlainSampleParallelThreads = 896;
// Radiance-cache render (kModeRenderNrc), training (kModeTrainNrc) or combined (kModeComboNrc)
// pass; `surfaces`: the instance that also traces the context's triangle meshes.
void launch_nrc_pass(const TraceParams& p, int mode, bool grid_majorant, bool surfaces, int grid_ctas, int threads,
                     size_t smem, cudaStream_t s);
const void* nrc_kernel_ptr(int mode, bool grid_majorant, bool surfaces);
// Jump table of sample-parallel streams first .. first + count - 1, computed on the device.
void launch_sample_jump_table(ulonglong2* out, uint32_t first, uint32_t count, cudaStream_t s);
void launch_finalize_mean(const double* sum, float* mean, uint32_t n_values, uint32_t samples, cudaStream_t s);
// Device frame counters of a context: [0] sample-parallel streams used since seeding, [1] samples
// in the accumulation. The launches of the plain and render paths read and advance them on the
// device, so a sequence of launches captured once in a CUDA graph renders new samples on replay.
void launch_sample_jump_table_dev(ulonglong2* out, const uint32_t* frame, uint32_t count, cudaStream_t s);
void launch_finalize_mean_dev(const double* sum, float* mean, uint32_t n_values, const uint32_t* frame, uint32_t spp,
                              cudaStream_t s);
void launch_frame_update(uint32_t* frame, uint32_t add_stream, bool set_accum, uint32_t value, cudaStream_t s);
void pool_majorants(const float* fine, int lx, int ly, int lz, float* out, int mx, int my, int mz, int factor,
                    cudaStream_t s);

}  // namespace vpt
