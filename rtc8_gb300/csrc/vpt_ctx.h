// Host-side state of a VptContext (device buffers and scene metadata).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <random>
#include <vector>

#include "../../include/rtc8_vpt.h"

namespace vpt {

struct TraceParams;
struct NrcBuffers;
struct Surfaces;

// Per-slot path state of the wavefront tracer (vpt_wavefront.cu), structure of arrays.
struct WfBuffers {
    uint32_t slots = 0;                // slots of the current launch (queue stride)
    uint32_t capacity = 0;             // allocated slots
    uint64_t* rng = nullptr;
    uint32_t* pixel = nullptr;
    uint32_t* sample = nullptr;
    uint32_t* path_length = nullptr;
    uint32_t* flags = nullptr;         // state | end code << 8 | segment flags
    uint2* rec = nullptr;              // primary / shadow lookups of the sample (decision log)
    float4* org = nullptr;             // vertex position, direction pdf
    float4* dir = nullptr;             // direction, initial importance
    float4* tp = nullptr;              // throughput, NEE area pdf
    float4* contrib = nullptr;         // contribution, NEE visibility
    float4* emit = nullptr;            // NEE emittance
    float4* seg0 = nullptr;            // segment eye, t
    float4* seg1 = nullptr;            // segment direction, t1
    int4* dda_i = nullptr;             // suspended segment: DDA cell, lookups so far
    float4* dda_f = nullptr;           // suspended segment: DDA tnext
    double* sum = nullptr;             // per-pixel streams: the pixel's sums (3 per slot)
    float4* mean = nullptr;            // per-pixel streams: the pixel's running mean
    uint32_t* track_queue = nullptr;   // 2 x slots
    uint32_t* event_queue = nullptr;   // 2 x slots
    uint32_t* count = nullptr;         // [0,1] tracking queues, [2,3] event queues, [4] tracking fetch
};

struct VptContextImpl {
    int32_t width = 0, height = 0;
    int device = 0, num_sms = 0;
    int32_t ctas_per_sm = 0, threads = 0, park_threshold = 0;
    int32_t leaf_stage_min = 0;         // > 0: per-warp leaf staging (vpt_set_leaf_staging)
    bool nrc_combined_pass = true;      // frame: first training pass and render samples in one launch

    // per pixel (renderer_main.cpp:80-129)
    uint64_t* d_rng = nullptr;
    double* d_sum = nullptr;
    float* d_mean = nullptr;
    uint32_t* d_rgba8 = nullptr;   // 8-bit output image of vpt_download_image_rgba8 (allocated on first use)
    uint32_t accum_samples = 0;
    uint32_t stream_samples = 0;   // samples ever traced since seeding (sample-parallel streams)
    uint32_t* d_frame = nullptr;   // device copy of {stream_samples, accum_samples} (authoritative)
    ulonglong2* d_jumps = nullptr; // per-launch PCG jump table of the sample-parallel streams
    uint32_t jump_capacity = 0;

    unsigned int* d_work = nullptr;
    unsigned long long* d_counters = nullptr;
    unsigned int* d_err = nullptr;
    unsigned int* d_scratch_u32 = nullptr;
    float* d_integral = nullptr;

    // density grid
    bool has_volume = false;
    float* d_dense = nullptr;
    int32_t* d_leaf_table = nullptr;
    float* d_leaf_values = nullptr;
    float* d_cell_maj = nullptr;
    float* d_maj = nullptr;          // majorant grid of the DDA (pooled cells)
    int32_t mx = 0, my = 0, mz = 0, maj_shift = 0;
    int32_t nx = 0, ny = 0, nz = 0, lx = 0, ly = 0, lz = 0;
    int64_t active_leaves = 0, total_leaves = 0;
    float global_majorant = 0, voxel_size = 1, inv_voxel_size = 1;
    float origin[3] = {0, 0, 0}, bbox_min[3] = {0, 0, 0}, bbox_max[3] = {0, 0, 0};
    float world_radius = 1;

    // environment
    float4* d_env = nullptr;
    float* d_mips = nullptr;
    int32_t env_w = 0, env_h = 0, map_w = 0, map_h = 0, num_mips = 0;
    int64_t mip_offset[16] = {};
    int64_t mip_total = 0;
    float imp_integral = 0;

    VptFrameParams frame{};
    bool has_frame = false;

    // neural-radiance-cache render/training buffers (allocated on first use)
    // wavefront tracer of the plain path (allocated on first use)
    int32_t tracker = 0;                // 0 = persistent megakernel, 1 = wavefront
    int32_t wf_slots_per_sm = 0, wf_pass_steps = 0, wf_track_ctas_per_sm = 0;
    WfBuffers wf;
    uint32_t* wf_pinned = nullptr;
    cudaEvent_t wf_events[8] = {};
    void release_wf();

    // surfaces (vpt_set_surfaces, vpt_surface.cu); device arrays owned through `surf_mem`
    Surfaces* surf = nullptr;            // host copy of the device view, nullptr = no surfaces
    std::vector<void*> surf_mem;
    uint32_t surf_nodes = 0, surf_emitters = 0;
    float surf_box_min[3] = {0, 0, 0}, surf_box_max[3] = {0, 0, 0};
    void release_surfaces();
    // World box and radius from the volume's box and the surfaces' box (compute_light_probs.cu:139-157).
    void update_world_box();
    float world_min[3] = {0, 0, 0}, world_max[3] = {0, 0, 0};

    NrcBuffers* nrc = nullptr;
    int32_t nrc_query_density = 0;
    float nrc_termination = 0.0f;          // 0 = the reference's pathTerminationFactor
    float nrc_train_termination = 0.0f;    // 0 = twice the render factor
    uint32_t nrc_buf_index = 1;            // the first training iteration uses buffer 0
    std::mt19937 nrc_offset_rng{72139121}; // perFrameRng (renderer_main.cpp:1500)
    void release_nrc();
};

int ctx_set_error(int code, const char* msg);
int fill_trace_params(VptContextImpl* c, TraceParams* tp);
int persistent_grid(VptContextImpl* c, int threads, const void* kernel, size_t smem);
// LCG jump (multiplier, increment) that advances a PCG32 state by `delta` draws.
void lcg_jump(uint64_t delta, uint64_t* mult, uint64_t* plus);
// Training-pass RNG states derived from the context's per-pixel states (no-op without cache buffers).
int nrc_reseed_train_rng(VptContextImpl* c);
// Jump table (A, C) of the next `count` sample-parallel streams (first = the device frame
// counter), enqueued on `s`; the caller advances the counter after its launch.
int upload_sample_jumps(VptContextImpl* c, uint32_t count, cudaStream_t s);
int generate_sky_texture(float4* out, int w, int h, const float* states, const float* solar, const float* cmf,
                         const float sun_dir[3], int include_disc);
const void* plain_kernel_ptr(bool grid_majorant, bool logged, bool sample_parallel, bool leaf_stage);
// Wavefront plain tracer: runs the passes of one launch on `s` (vpt_wavefront.cu).
int wf_run(VptContextImpl* c, const TraceParams& tp, bool grid_majorant, size_t smem, cudaStream_t s);
int wf_ensure(VptContextImpl* c, uint32_t slots);
const void* wf_track_kernel_ptr(bool grid_majorant);
// Tone map + 8-bit conversion of the mean image (vpt_post.cu).
int launch_tonemap(VptContextImpl* c, cudaStream_t s, float brightness, uint32_t flags, float* rgba32, uint32_t* rgba8);
// Uploads a flattened sparse grid (leaf table over the extent starting at index `lo`, leaves in
// slot order with their extent-relative origins) and derives its majorants (vpt_nvdb.cu).
int upload_sparse_grid(VptContextImpl* c, const std::vector<int32_t>& table, int32_t lx, int32_t ly, int32_t lz,
                       const std::vector<int32_t>& origins, const float* values, int64_t slots, const int32_t lo[3],
                       const VptNanoVdbInfo& info);

}  // namespace vpt

// The opaque handle of the C ABI.
struct VptContext : vpt::VptContextImpl {};
