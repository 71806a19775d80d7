// Persistent megakernel for the plain volumetric path tracer (the reference's pathTrace
// ray-generation program, renderer/gpu_kernels/optix_pathtracing_kernels.cu:31-434 with
// withNRC = generateTrainingData = false, for volume-only scenes).
//
// GB300 layout: one resident set of CTAs per SM pulls work items from a global counter (path
// regeneration: a lane that finishes a path starts the next one at once). A work item is a
// pixel (reference streams: its samples are traced in order so the pixel's PCG32 stream
// advances exactly as in the reference) or one (pixel, sample) pair (sample-parallel streams).
// Each loop iteration first lets every lane run its cheap, divergent event logic (camera ray,
// vertex, Russian roulette, NEE set-up, phase sampling, accumulation, a bounded number of
// majorant-grid cell steps) until it needs a density value, then all lanes perform their grid
// lookups together, so the dominant gathers of delta and ratio tracking run converged. The
// majorant grid is staged in shared memory when it fits.
#include "vpt_ctx.h"
#include "vpt_tracer.cuh"

namespace vpt {
namespace {

enum : uint32_t {
    ST_FETCH = 0,    // get the next work item
    ST_CAMERA,       // start a sample: camera ray
    ST_SEGMENT,      // start a primary segment: ++pathLength, clip
    ST_STEP,         // advance the current segment to its next lookup
    ST_VERTEX,       // primary collision: RR, NEE set-up
    ST_NEE_DONE,     // shadow segment finished: NEE contribution, phase sampling
    ST_ESCAPE,       // primary segment left the grid
    ST_END_SAMPLE,   // accumulate, next sample or next item
    ST_DONE,
    ST_SURFACE,      // surface scenes: the primary segment ended on a triangle
    ST_NEE_SETUP,    // surface scenes: light sample and shadow ray of the current vertex
};

enum : uint32_t {
    END_ESCAPE = 1,
    END_RR = 2,
    END_PDF_ZERO = 3,
    END_MAX_BOUNCES = 4,
    END_STEP_CAP = 5,
    END_CACHE = 6,       // radiance-cache passes: ended with a cache query
    END_TRAIN_FULL = 7,  // training pass: the training-vertex buffer was full
};

// Limits that apply even when the caller disables the configurable caps, so that no input
// (zero or non-finite majorants, albedo 1 in a huge medium) can keep a launch running forever.
constexpr uint32_t kHardStepCap = 1u << 24;
constexpr uint32_t kHardVertexCap = 1u << 16;
// Majorant-grid cells a lane crosses per tracking iteration before yielding to the warp. With
// a pixel's samples traced consecutively (C2 / C5 ms per 16-spp launch, radiance-cache frame ms):
// 8 -> 29.3 / 53.7 / 5.02, 16 -> 29.9 / 54.5 / -, 32 -> 29.5 / 54.6 / -; the radiance-cache passes
// at 4 / 8 / 16: 5.08 / 5.02 / 5.01. Earlier, with the samples of all pixels interleaved (M paths/s):
// 4 -> 454 / 927, 8 -> 471 / 979, 16 -> 480 / 977, 32 -> 481 / 974 (1 -> 4 had raised C2 by 12% with
// IEEE division and libm-accurate functions).
constexpr int kCellStepsPerPass = 8;
constexpr int kNrcCellStepsPerPass = 8;
constexpr int kSurfCellStepsPerPass = 16;
// Parked lanes of a warp that trigger a joint event phase. Plain tracer, C2 / C5 / C1 ms per
// 16-spp launch with a pixel's samples consecutive: 12 -> 30.6 / 55.4 / 1.13, 16 -> 29.6 / 54.6 /
// 1.15, 20 -> 29.8 / 55.4 / 1.17, 24 -> 31.2 / 58.2 / 1.17, 28 -> 33.6 / 62.1 / 1.15 (with the samples
// of all pixels interleaved 20 was best); the radiance-cache passes (shorter paths, more event
// work per path) are fastest at 24 (frame 5.05 ms; 16 / 20 / 28 / 32: 5.31 / 5.09 / 5.06 / 5.23).
constexpr int kParkThreshold = 16;
// The surface tracer keeps the values it was tuned with (park threshold 20, 16 cells per step:
// room scene 512^2 x 16 spp 92.8 ms per launch against 96.7 ms with the volume tracer's 16 and 8).
constexpr int kSurfParkThreshold = 20;
constexpr int kNrcParkThreshold = 24;
// Resident CTAs per SM the register allocation is bounded for (CTAs of 128 threads unless noted).
// The plain tracer on sample-parallel streams holds its state in 72 registers at 28 warps per SM
// (1024^2 sparse 512^3 with 128-thread CTAs: 261 / 284 / 295 / 283 M paths/s at 5 / 6 / 7 / 8 per
// SM). It runs them as ONE CTA of kPlainSampleParallelThreads = 896 threads per SM: one copy of
// the staged majorant grid per SM instead of seven leaves more of the SM's L1 to the density
// gathers (C2 / C5 / C1 per 16-spp launch: 35.0 / 68.4 / 1.17 ms as 7 x 128, 34.5 / 67.8 / 1.14
// as 2 x 448, 34.0 / 67.0 / 1.13 as 1 x 896; 3 x 256 and 2 x 384, with more registers, slower).
// Per-pixel streams (and the logged parity kernels) carry per-lane FP64 sums and stay at 5 CTAs
// of 128, where they need no spills. The radiance-cache passes measured best at 7 x 128 (8 equal)
// and better still as one 896-thread CTA per SM (256^2 frame: render pass 4.53 -> 4.44 ms, frame
// 6.28 -> 6.13 ms); over meshes they keep CTAs of 128 (kSurfCtasPerSm).
constexpr int kPlainCtasPerSm = 1;
constexpr int kPlainPerPixelCtasPerSm = 5;
constexpr int kNrcCtasPerSm = 1;
// The surface tracer carries the hit, the light sample's geometry and a BVH stack per lane; it
// is latency-bound (every vertex traverses the BVH twice with divergent loops), and occupancy wins
// over register spills: room scene 512^2 x 16 spp, 4 / 6 / 8 / 10 / 12 / 16 CTAs per SM ->
// 176 / 151 / 137 / 132 / 128 / 121 ms per launch through the BVH (with the flat triangle loop:
// 8 / 12 / 16 -> 110.7 / 102.4 / 96.7 ms; the same 2048 threads as 2 x 1024, 4 x 512 or 8 x 256
// threads within 1%).
constexpr int kSurfCtasPerSm = 16;

struct DdaState {
    int cell[3];
    int step[3];
    float tnext[3], tdelta[3];
};

// Majorant-grid DDA in index space. Cells are 2^maj_shift voxels wide; shared definition with
// the oracle's restatement (overshooting a cell's exit restarts sampling at the exit).
__device__ __forceinline__ void dda_init(const Grid& g, V3 eye, V3 dir, float t, DdaState* d) {
    float o[3] = {(eye.x - g.origin[0]) * g.inv_voxel_size, (eye.y - g.origin[1]) * g.inv_voxel_size,
                  (eye.z - g.origin[2]) * g.inv_voxel_size};
    float dd[3] = {dir.x * g.inv_voxel_size, dir.y * g.inv_voxel_size, dir.z * g.inv_voxel_size};
    int cdim[3] = {g.mx, g.my, g.mz};
    const float size = static_cast<float>(1 << g.maj_shift);
    const float inv_size = 1.0f / size;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float p = o[a] + dd[a] * t;
        int c = static_cast<int>(floorf(p * inv_size));
        c = min(max(c, 0), cdim[a] - 1);
        d->cell[a] = c;
        if (dd[a] > 0) {
            d->step[a] = 1;
            d->tnext[a] = ((c + 1) * size - o[a]) / dd[a];
            d->tdelta[a] = size / dd[a];
        } else if (dd[a] < 0) {
            d->step[a] = -1;
            d->tnext[a] = (c * size - o[a]) / dd[a];
            d->tdelta[a] = -size / dd[a];
        } else {
            d->step[a] = 0;
            d->tnext[a] = INFINITY;
            d->tdelta[a] = INFINITY;
        }
    }
}

__device__ __forceinline__ float cell_maj(const float* maj, const Grid& g, const DdaState& d) {
    return maj[(d.cell[0] * g.my + d.cell[1]) * g.mz + d.cell[2]];
}

enum : int { PASS_LOOKUP = 0, PASS_YIELD = 1, PASS_END = 2 };

// One tracking pass of a segment from (t, texit, maj, dda): a free-flight distance
// (optix_pathtracing_kernels.cu:113-118 / renderer_kernel_common.h:374-378), with the majorant
// grid sampled within the current cell, where an overshoot of the cell's exit restarts at the
// exit (memoryless) and empty cells are crossed without draws, at most kCells crossings per
// pass. PASS_LOOKUP leaves t at the tentative collision; PASS_END means the segment
// is over (also on a NaN distance); PASS_YIELD means the pass crossed its cells without one.
// The sign of a direction component: the DDA step along that axis (dda_init derives it from the
// same sign, the index-space direction being the world direction times a positive scale).
__device__ __forceinline__ int step_of(float d) { return d > 0 ? 1 : (d < 0 ? -1 : 0); }

template <bool kGridMajorant, int kCells>
__device__ __forceinline__ int track_pass(const Grid& g, const float* maj_grid, float density_coeff, float t1, V3 dir,
                                          Pcg32& rng, float& t, float& texit, float& maj, DdaState& dda,
                                          uint32_t& n_cells) {
    if constexpr (!kGridMajorant) {
        t += -logf(1.0f - rng.uniform()) / maj;
        return (t <= t1) ? PASS_LOOKUP : PASS_END;
    } else {
        for (int c = 0; c < kCells; ++c) {
            if (maj > 0) {
                const float tt = t + -logf(1.0f - rng.uniform()) / maj;
                if (tt < texit) {
                    t = tt;
                    return PASS_LOOKUP;
                }
            }
            t = texit;
            if (texit >= t1) return PASS_END;
            // Advance along the axis whose boundary comes first (x, then y, then z on ties);
            // written with selects so the DDA state stays in registers.
            const bool ax0 = dda.tnext[0] <= dda.tnext[1] && dda.tnext[0] <= dda.tnext[2];
            const bool ax1 = !ax0 && dda.tnext[1] <= dda.tnext[2];
            const bool ax2 = !ax0 && !ax1;
            if (ax0) dda.cell[0] += step_of(dir.x);
            if (ax1) dda.cell[1] += step_of(dir.y);
            if (ax2) dda.cell[2] += step_of(dir.z);
            ++n_cells;
            if (dda.cell[0] < 0 || dda.cell[0] >= g.mx || dda.cell[1] < 0 || dda.cell[1] >= g.my || dda.cell[2] < 0 ||
                dda.cell[2] >= g.mz) {
                t = t1;
                return PASS_END;
            }
            if (ax0) dda.tnext[0] += dda.tdelta[0];
            if (ax1) dda.tnext[1] += dda.tdelta[1];
            if (ax2) dda.tnext[2] += dda.tdelta[2];
            texit = fminf(fminf(dda.tnext[0], dda.tnext[1]), fminf(dda.tnext[2], t1));
            maj = density_coeff * cell_maj(maj_grid, g, dda);
        }
        return PASS_YIELD;
    }
}

// createRadianceQuery (optix_pathtracing_kernels.cu:14-29) for an in-medium vertex: position in
// the world box (basic_types.h:2835-2838), normal = vOut as toPolarYUp outputs (the first slot
// holds acos(y), the second the azimuth), roughness, diffuse = albedo, specular = 0.
__device__ __forceinline__ void write_query(float* q, V3 pos, V3 vout, float roughness, float albedo, V3 wmin, V3 wmax) {
    V3 d = wmax - wmin, r = pos - wmin;
    float a, b;
    to_polar_yup_sel(vout, &a, &b);
    float2* p = reinterpret_cast<float2*>(q);
    p[0] = make_float2(d.x != 0 ? r.x / d.x : 0.0f, d.y != 0 ? r.y / d.y : 0.0f);
    p[1] = make_float2(d.z != 0 ? r.z / d.z : 0.0f, a);
    p[2] = make_float2(b, a);
    p[3] = make_float2(b, roughness);
    p[4] = make_float2(albedo, albedo);
    p[5] = make_float2(albedo, 0.0f);
    p[6] = make_float2(0.0f, 0.0f);
}

// RadianceQuery of a surface vertex (optix_pathtracing_kernels.cu:14-29 with the BSDF's
// getSurfaceParameters, common_renderer_types.h:1491-1496 Lambert, 1671-1677 dichromatic):
// position in the world box, the shading normal and vOut as toPolarYUp outputs, roughness,
// diffuse and specular reflectance of the material.
__device__ __forceinline__ void write_query_surface(float* q, V3 pos, V3 normal, V3 vout, const SurfMaterial& m, V3 wmin,
                                                    V3 wmax) {
    V3 d = wmax - wmin, r = pos - wmin;
    float na, nb, va, vb;
    to_polar_yup_sel(normal, &na, &nb);
    to_polar_yup_sel(vout, &va, &vb);
    float2* p = reinterpret_cast<float2*>(q);
    p[0] = make_float2(d.x != 0 ? r.x / d.x : 0.0f, d.y != 0 ? r.y / d.y : 0.0f);
    p[1] = make_float2(d.z != 0 ? r.z / d.z : 0.0f, na);
    p[2] = make_float2(nb, va);
    p[3] = make_float2(vb, m.roughness);
    p[4] = make_float2(m.diffuse[0], m.diffuse[1]);
    p[5] = make_float2(m.diffuse[2], m.specular[0]);
    p[6] = make_float2(m.specular[1], m.specular[2]);
}

// Work order of the training pass: item -> pixel of the training image, class by class, where
// the class of a pixel is (its position in the 4x4 tile + offset) % 16 and class 0 holds the
// unbiased suffixes (optix_pathtracing_kernels.cu:60-66). The long unbiased paths thus gather in
// the first warps and CTAs, and the CTAs of the short biased suffixes retire early, freeing their
// SM slots for the render pass that runs concurrently. Records stay at the reference's pixel
// index; only the order in which the pixels are traced changes.
__device__ __forceinline__ void train_item_to_pixel(uint32_t item, uint32_t w, uint32_t h, uint32_t offset,
                                                    uint32_t* px, uint32_t* py) {
    const uint32_t off = offset % 16;
    for (uint32_t k = 0; k < 16; ++k) {
        const uint32_t p = (k + 16 - off) % 16;  // tile position with (p + offset) % 16 == k
        const uint32_t a = p % 4, b = p / 4;
        const uint32_t cx = w > a ? (w - a + 3) / 4 : 0, cy = h > b ? (h - b + 3) / 4 : 0;
        const uint32_t n = cx * cy;
        if (item < n) {
            *px = a + 4 * (item % cx);
            *py = b + 4 * (item / cx);
            return;
        }
        item -= n;
    }
    *px = 0;  // not reached for item < w * h
    *py = 0;
}

// kMode: kModePlain (pathTrace), kModeRenderNrc (pathTraceWithNRC) or kModeTrainNrc
// (generateTrainingData), optix_pathtracing_kernels.cu:438-448.
// kStreams: the RNG stream layout the kernel is compiled for (kStreamsPerPixel,
// kStreamsSampleParallel), or kStreamsRuntime to follow TraceParams::stream_mode. A fixed layout
// drops the other layout's state (the per-lane FP64 sums and running mean of per-pixel streams)
// from the register allocation.
constexpr int kStreamsPerPixel = 0, kStreamsSampleParallel = 1, kStreamsRuntime = 2;

// kStage: per-warp leaf staging in shared memory (sample_trilinear_staged; TraceParams::
// leaf_stage_min lanes in one leaf trigger a bulk copy of that leaf).
// kSurfaces: the scene has triangle meshes (TraceParams::surf): every primary segment first
// finds its closest triangle, volume tracking stops there, surface vertices scatter by their
// BSDF, NEE also samples the emitting triangles and shadow rays test the triangles for
// visibility (optix_pathtracing_kernels.cu:84-96, 176-195, 216-239, 268-275, 340-356;
// renderer_kernel_common.h:72-124, 146-403), in the plain and the radiance-cache modes.
template <bool kGridMajorant, bool kLog, int kMode, int kStreams = kStreamsRuntime, bool kStage = false,
          bool kSurfaces = false>
__global__ void __launch_bounds__(((kMode == kModePlain && kStreams == kStreamsSampleParallel) || kMode != kModePlain) && !kSurfaces
                                      ? kPlainSampleParallelThreads
                                      : 128,
                                  kSurfaces                              ? kSurfCtasPerSm
                                       : kMode != kModePlain                  ? kNrcCtasPerSm
                                       : kStreams == kStreamsSampleParallel ? kPlainCtasPerSm
                                                                            : kPlainPerPixelCtasPerSm)
    plain_trace_kernel(const TraceParams P) {
    static_assert(!kSurfaces || !kStage, "surfaces: no leaf staging");
    const bool sample_parallel = kStreams == kStreamsRuntime ? P.stream_mode == 1 : kStreams == kStreamsSampleParallel;
    extern __shared__ __align__(128) float s_maj[];
    const Grid& g = P.grid;
    const float* maj_grid = g.maj;
    if constexpr (kGridMajorant) {
        if (P.maj_in_smem) {
            const int cells = g.mx * g.my * g.mz;
            for (int i = threadIdx.x; i < cells; i += blockDim.x) s_maj[i] = g.maj[i];
            __syncthreads();
            maj_grid = s_maj;
        }
    }
    LeafStage stage{nullptr, nullptr, -1, -1, 0u};
    bool stage_timed_out = false;
    if constexpr (kStage) {
        // After the staged majorant grid: the warps' leaf buffers, then their mbarriers.
        const size_t maj_bytes = P.maj_in_smem ? static_cast<size_t>(g.mx) * g.my * g.mz * sizeof(float) : 0;
        unsigned char* area = reinterpret_cast<unsigned char*>(s_maj) + (maj_bytes + 127) / 128 * 128;
        const int warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
        stage.values = reinterpret_cast<float*>(area + static_cast<size_t>(warp) * kLeafBytes);
        stage.bar = reinterpret_cast<uint64_t*>(area + static_cast<size_t>(warps) * kLeafBytes) + warp;
        if ((threadIdx.x & 31) == 0) stage_bar_init(stage.bar);
        __syncwarp();
    }
    const uint32_t num_pixels = static_cast<uint32_t>(P.width) * static_cast<uint32_t>(P.height);
    const float global_maj = P.density_coeff * g.global_majorant;
    const uint32_t step_cap = P.max_steps > 0 ? static_cast<uint32_t>(P.max_steps) : kHardStepCap;
    const int park_threshold =
        P.park_threshold > 0 ? P.park_threshold
                             : (kMode == kModePlain ? (kSurfaces ? kSurfParkThreshold : kParkThreshold) : kNrcParkThreshold);
    const V3 bmin = v3(g.bbox_min[0], g.bbox_min[1], g.bbox_min[2]);
    const V3 bmax = v3(g.bbox_max[0], g.bbox_max[1], g.bbox_max[2]);
    // Sensor height of the launch's camera (optix_pathtracing_kernels.cu:43-55); the rest of the
    // camera set-up is a few multiplies per sample, cheaper than keeping it in registers.
    const float cam_vh = 2 * tanf(P.cam_fovy * 0.5f);

    uint32_t st = ST_FETCH;
    uint32_t pixel = 0, sample = 0;
    Pcg32 rng{0};
    double sum_r = 0, sum_g = 0, sum_b = 0;
    RGB mean = rgb(0, 0, 0);

    // per-sample state
    V3 origin = v3(0, 0, 0), dir = v3(0, 0, 1);
    float dir_pdf = 1.0f, init_importance = 1.0f;
    RGB throughput = rgb(0, 0, 0), contribution = rgb(0, 0, 0);
    uint32_t path_length = 0, end_code = 0;
    uint32_t rec_primary = 0, rec_shadow = 0;

    // current segment
    bool shadow = false;
    // The segment's eye and direction are not stored: a primary segment starts at the path's
    // origin along its direction, a shadow segment at origin + trace_len * light_dir towards
    // -light_dir (both unchanged while the segment is tracked).
    const float trace_len = 2 * P.world_radius;
    float t = 0, t1 = 0, maj = global_maj, texit = 0;
    uint32_t seg_steps = 0;
    DdaState dda;

    // NEE in flight
    V3 light_dir = v3(0, 1, 0);
    RGB emittance = rgb(0, 0, 0);
    float area_pdf = 1.0f, vis = 1.0f;
    bool pick_sun = false;

    // Surface scenes: the current primary segment's closest triangle (~0u = none), whether the
    // current vertex is on a surface, and the shadow ray of a light sample (its origin, the
    // light-side cosine over the length and the squared distance; 1 and 1 for the environment).
    uint32_t hit_tri = ~0u;
    float hit_b1 = 0.0f, hit_b2 = 0.0f;
    bool at_surface = false;
    V3 shadow_eye = v3(0, 0, 0);
    float nee_lp_cos = 1.0f, nee_dist2 = 1.0f;

    // Per-lane work counters (32-bit: a lane does far fewer than 2^32 steps in a launch), summed
    // over the warp in 64 bits at the end.
    uint32_t n_lookups = 0, n_vertices = 0, n_samples = 0, n_cells = 0;
    unsigned int err = 0;
    LeafCache leaf_cache;

    // Radiance-cache passes: one sample per pixel of the pass image (the training image has the
    // adaptive size prepared on the device), RNG states of the full image's per-pixel buffer.
    // kModeComboNrc runs one training pass and one batched render pass as ONE launch: work items
    // [0, num_train) are the training pixels, the rest the render samples, so lanes that finish
    // their training suffix go on with render samples and no SM slot idles behind the longest
    // suffixes. is_train tells a lane which kind of item it traces.
    constexpr bool kNrc = kMode != kModePlain;
    constexpr bool kCombo = kMode == kModeComboNrc;
    constexpr bool kMayTrain = kMode == kModeTrainNrc || kCombo;
    bool is_train = kMode == kModeTrainNrc;
    // Training image of the pass (the adaptive size prepared on the device). The pass image
    // size, the item counts and the state buffer a sample continues are derived from these and
    // `is_train` where needed rather than held in registers.
    // A combined launch traces P.num_train_sets training images (the frame's training
    // iterations), set k from the arrays of P.train_sets[k]; tset is the set of the lane's item.
    uint32_t train_w = 0, train_h = 0, num_train = 0, tset = 0;
    auto set_buf = [&](uint32_t k) -> uint32_t { return (P.train_bufs >> k) & 1u; };
    auto set_w = [&](uint32_t k) -> uint32_t {
        return min(P.train_sets[k].counters[2 + 2 * set_buf(k)], static_cast<uint32_t>(P.width));
    };
    auto set_h = [&](uint32_t k) -> uint32_t {
        return min(P.train_sets[k].counters[3 + 2 * set_buf(k)], static_cast<uint32_t>(P.height));
    };
    if constexpr (kMode == kModeTrainNrc) {
        train_w = min(P.nrc.counters[2 + 2 * P.nrc_buf], static_cast<uint32_t>(P.width));
        train_h = min(P.nrc.counters[3 + 2 * P.nrc_buf], static_cast<uint32_t>(P.height));
        num_train = min(train_w * train_h, num_pixels);
    } else if constexpr (kCombo) {
        for (uint32_t k = 0; k < P.num_train_sets; ++k) num_train += min(set_w(k) * set_h(k), num_pixels);
    }
    // The arrays a training item writes: its set's in a combined launch, the pass's own otherwise.
    auto tr_counters = [&]() -> uint32_t* {
        if constexpr (kCombo) return P.train_sets[tset].counters;
        else return P.nrc.counters;
    };
    auto tr_buf = [&]() -> uint32_t {
        if constexpr (kCombo) return set_buf(tset);
        else return P.nrc_buf;
    };
    auto tr_vertex = [&]() -> TrainVertexInfo* {
        if constexpr (kCombo) return P.train_sets[tset].vertex;
        else return P.nrc.train_vertex;
    };
    auto tr_query0 = [&]() -> float* {
        if constexpr (kCombo) return P.train_sets[tset].query0;
        else return P.nrc.train_query[0];
    };
    auto tr_target0 = [&]() -> float* {
        if constexpr (kCombo) return P.train_sets[tset].target0;
        else return P.nrc.train_target[0];
    };
    auto tr_end_query = [&]() -> float* {
        if constexpr (kCombo) return P.train_sets[tset].end_query;
        else return P.nrc.train_end_query;
    };
    auto tr_suffix = [&]() -> uint32_t* {
        if constexpr (kCombo) return P.train_sets[tset].suffix;
        else return P.nrc.train_suffix;
    };
    uint32_t slot = 0;  // record index of the current sample in the pass buffers
    const float term_factor = P.nrc_termination > 0 ? P.nrc_termination : kPathTerminationFactor;
    // Biased training suffixes end at twice the render factor (optix_pathtracing_kernels.cu:
    // 284-285) unless a separate training factor is set.
    const float train_term_factor = P.nrc_train_termination > 0 ? P.nrc_train_termination : 2 * term_factor;
    // Radiance queries locate positions in the world box (worldDimInfo.aabb,
    // optix_pathtracing_kernels.cu:19), which is the volume's box unless the scene has meshes.
    const V3 wmin = kSurfaces ? v3(P.world_min[0], P.world_min[1], P.world_min[2]) : bmin;
    const V3 wmax = kSurfaces ? v3(P.world_max[0], P.world_max[1], P.world_max[2]) : bmax;
    uint32_t rng_index = 0;
    float primary_spread = 0.0f, sqrt_spread = 0.0f, last_density = 0.0f;
    uint32_t prev_vertex = kInvalidVertex;
    RGB nee_value = rgb(0, 0, 0);
    bool unbiased = false, terminal_written = false;

    // NEE set-up of a surface scene at the vertex `origin` (renderer_kernel_common.h:297-358):
    // the environment group (image or sky, and the sun) against the emitting triangles with
    // probToSampleEnvLight, the light sample, the triangles' visibility test from the light
    // towards the vertex, then the shadow segment through the volume.
    auto surf_nee_setup = [&]() {
        float u_light = rng.uniform();
        const float u0 = rng.uniform();
        const float u1 = rng.uniform();
        pick_sun = false;
        const bool areas = P.surf.inst_integral > 0.0f;
        const bool env_group = P.env_enabled || P.sun.enabled;
        bool select_env = false;
        float type_prob = 1.0f;
        if (env_group) {
            if (areas) {
                if (u_light < kProbEnvLight) {
                    type_prob = kProbEnvLight;
                    u_light /= type_prob;
                    select_env = true;
                } else {
                    type_prob = 1.0f - kProbEnvLight;
                    u_light = (u_light - kProbEnvLight) / type_prob;
                }
            } else {
                select_env = true;
            }
        }
        vis = 0.0f;
        nee_lp_cos = 1.0f;
        nee_dist2 = 1.0f;
        bool have_light = env_group || areas;
        V3 sdir = v3(0, 0, 1);
        float trace_length = trace_len;
        if (have_light && select_env) {
            float light_prob = 1.0f;
            if (P.sun.enabled && P.env_enabled) {
                if (u_light < P.sun.select_prob) {
                    pick_sun = true;
                    light_prob = P.sun.select_prob;
                } else {
                    light_prob = 1.0f - P.sun.select_prob;
                }
            } else if (P.sun.enabled) {
                pick_sun = true;
            }
            if (pick_sun) {
                light_dir = v3(P.sun.dir[0], P.sun.dir[1], P.sun.dir[2]);
                emittance = rgb(P.sun.irradiance[0], P.sun.irradiance[1], P.sun.irradiance[2]);
                area_pdf = light_prob;
            } else {
                float pdf;
                const RGB radiance = env_sample(P.env, u0, u1, &light_dir, &pdf);
                emittance = kPi * radiance;
                area_pdf = pdf;
                if (area_pdf == 0.0f) have_light = false;
                area_pdf *= light_prob;
            }
            if (have_light) {
                area_pdf *= type_prob;
                sdir = -light_dir;
                nee_lp_cos = dot(sdir, -light_dir);
                if (nee_lp_cos <= 0.0f) have_light = false;
                shadow_eye = origin + trace_len * light_dir;
            }
        } else if (have_light) {
            const AreaSample as = sample_area_light(P.surf, u_light, u0, u1);
            if (as.area_pdf == 0.0f) {
                have_light = false;
            } else {
                area_pdf = as.area_pdf * type_prob;
                emittance = as.emittance;
                sdir = origin - as.pos;
                const float lp_cos = dot(sdir, as.normal);
                if (lp_cos <= 0.0f) {
                    have_light = false;
                } else {
                    shadow_eye = offset_ray_origin(as.pos, as.normal);
                    sdir = origin - shadow_eye;
                    nee_dist2 = dot(sdir, sdir);
                    trace_length = sqrtf(nee_dist2);
                    sdir = sdir * (1.0f / trace_length);
                    nee_lp_cos = lp_cos / trace_length;
                    light_dir = -sdir;
                }
            }
        }
        if (!have_light) {
            st = ST_NEE_DONE;  // vis = 0: no contribution
            return;
        }
        bool overflow = false;
        const bool blocked = bvh_any(P.surf, shadow_eye, sdir, 0.0f, trace_length * 0.9999f, &overflow);
        if (overflow) err |= VPT_DEVERR_BVH_STACK;
        if (blocked) {
            st = ST_NEE_DONE;
            return;
        }
        vis = 1.0f;
        float a, b;
        if (P.volume_enabled && clip_ray(bmin, bmax, shadow_eye, sdir, 0.0f, trace_length, &a, &b)) {
            shadow = true;
            t = fmaxf(0.0f, a);
            t1 = b;
            seg_steps = 0;
            if constexpr (kGridMajorant) {
                dda_init(g, shadow_eye, sdir, t, &dda);
                texit = fminf(fminf(dda.tnext[0], dda.tnext[1]), fminf(dda.tnext[2], t1));
                maj = P.density_coeff * cell_maj(maj_grid, g, dda);
            } else {
                maj = global_maj;
            }
            st = ST_STEP;
        } else {
            st = ST_NEE_DONE;
        }
    };

    // The path ends at a vertex whose cache query was just written (optix_pathtracing_kernels.cu
    // :307-330): the training suffix's terminal record, or the render path's terminal info and,
    // when the render queries are listed, its slot in the inference list.
    auto end_with_query = [&]() {
        if (kMayTrain && is_train) {
            tr_suffix()[slot] = pack_suffix(prev_vertex, 1, path_length, unbiased ? 1 : 0);
        } else {
            TerminalInfo ti;
            ti.tp[0] = throughput.r;
            ti.tp[1] = throughput.g;
            ti.tp[2] = throughput.b;
            ti.bits = 1u | ((path_length & 0xFFu) << 1);
            P.nrc.infer_terminal[slot] = ti;
            if (P.nrc.infer_index) {
                // List the slot for the inference (one atomic per converged group).
                const uint32_t m = __activemask();
                const int leader = __ffs(m) - 1;
                const uint32_t lane = threadIdx.x & 31;
                uint32_t base = 0;
                if (static_cast<int>(lane) == leader) base = atomicAdd(P.nrc.counters + 8, __popc(m));
                base = __shfl_sync(m, base, leader);
                P.nrc.infer_index[base + __popc(m & ((1u << lane) - 1u))] = slot;
            }
        }
        terminal_written = true;
        end_code = END_CACHE;
        st = ST_END_SAMPLE;
    };

    while (true) {
        // Warp-level event batching: lanes whose path reached an event (segment end, collision,
        // new sample) park until at least kParkThreshold lanes of the warp are parked, or no lane
        // is tracking any more; then all parked lanes run their event logic together. In between,
        // the tracking lanes advance one step per iteration (a density lookup or one DDA cell).
        const bool tracking = st == ST_STEP;
        const uint32_t ev_mask = __ballot_sync(0xffffffffu, !tracking && st != ST_DONE);
        const uint32_t tr_mask = __ballot_sync(0xffffffffu, tracking);
        if ((ev_mask | tr_mask) == 0) break;
        const bool event_phase = ev_mask != 0 && (tr_mask == 0 || __popc(ev_mask) >= park_threshold);
        bool need_lookup = false, yield = false;
        V3 lookup_pos = v3(0, 0, 0);
        while (!need_lookup && !yield && st != ST_DONE && (event_phase ? st != ST_STEP : st == ST_STEP)) {
            switch (st) {
            case ST_FETCH: {
                // Warp-aggregated fetch: one atomic for all lanes of the warp that need work now.
                const uint32_t need = __activemask();
                const int leader = __ffs(need) - 1;
                const uint32_t lane = threadIdx.x & 31;
                uint32_t base = 0;
                if (static_cast<int>(lane) == leader) base = atomicAdd(P.work_counter, __popc(need));
                base = __shfl_sync(need, base, leader);
                const uint32_t item = base + __popc(need & ((1u << lane) - 1u));
                if constexpr (kNrc) {
                    // Sample-parallel streams: P.spp samples per pixel in one render pass, each
                    // its own work item and record slot (sample-major: slot = sample * pixels + pixel).
                    uint32_t num_items = num_pixels;
                    if constexpr (kMode == kModeTrainNrc) {
                        num_items = num_train;
                    } else {
                        if (sample_parallel) num_items = num_pixels * P.spp;
                        if constexpr (kCombo) num_items += num_train;
                    }
                    if (item >= num_items) {
                        st = ST_DONE;
                        break;
                    }
                    if constexpr (kCombo) is_train = item < num_train;
                    sample = 0;
                    if (kMayTrain && is_train) {
                        uint32_t px, py, local = item, tw = train_w, th = train_h;
                        if constexpr (kCombo) {
                            tset = 0;
                            while (tset + 1 < P.num_train_sets) {
                                const uint32_t n = min(set_w(tset) * set_h(tset), num_pixels);
                                if (local < n) break;
                                local -= n;
                                ++tset;
                            }
                            tw = set_w(tset);
                            th = set_h(tset);
                        }
                        const uint32_t offset = tr_counters()[6];
                        train_item_to_pixel(local, tw, th, offset, &px, &py);
                        pixel = py * tw + px;  // linear index in the training image
                        slot = pixel;
                        rng_index = py * static_cast<uint32_t>(P.width) + px;
                        if constexpr (kCombo)
                            rng.state = P.train_sets[tset].rng[rng_index];
                        else
                            rng.state = P.rng[rng_index];
                        // optix_pathtracing_kernels.cu:60-66: one unbiased suffix per 4x4 tile.
                        const uint32_t tile_index = (py % 4) * 4 + (px % 4);
                        unbiased = (tile_index + offset) % 16 == 0;
                        st = ST_CAMERA;
                        break;
                    }
                    const uint32_t r = kCombo ? item - num_train : item;
                    slot = r;
                    if (sample_parallel) {
                        // Traced pixel by pixel like the plain passes (render pass at 256^2 x 128
                        // spp: 4.44 -> 3.75 ms); the records stay sample-major.
                        pixel = r / P.spp;
                        sample = r % P.spp;
                        slot = sample * num_pixels + pixel;
                        const ulonglong2 jump = P.sample_jumps[sample];
                        rng.state = jump.x * P.rng[pixel] + jump.y;
                    } else {
                        pixel = r;
                        rng_index = r;
                        rng.state = P.rng[rng_index];
                    }
                    st = ST_CAMERA;
                    break;
                }
                if (sample_parallel) {
                    // One (pixel, sample) per work item, the spp samples of a pixel consecutive: the
                    // lanes of a warp (and the warps of an SM) trace the same pixel's primary rays
                    // through the same leaves, which the L1 and the warps' convergence reward (C2 /
                    // C5 per 16-spp launch 34.0 / 67.1 ms with samples of all pixels interleaved,
                    // 29.8 / 55.6 ms pixel by pixel; groups of 2 / 4 / 8 samples in between).
                    if (item >= num_pixels * P.spp) {
                        st = ST_DONE;
                        break;
                    }
                    pixel = item / P.spp;
                    sample = item % P.spp;
                    // Sample (stream_base + sample) starts (stream_base + sample) * 2^40 draws into
                    // the pixel's stream: state = A * seed + C with the launch's jump table.
                    const ulonglong2 jump = P.sample_jumps[sample];
                    rng.state = jump.x * P.rng[pixel] + jump.y;
                    st = ST_CAMERA;
                    break;
                }
                pixel = item;
                if (pixel >= num_pixels) {
                    st = ST_DONE;
                    break;
                }
                rng.state = P.rng[pixel];
                sum_r = sum_g = sum_b = 0;
                if (P.accum_base > 0) {
                    mean = rgb(P.mean_rgb[3 * pixel], P.mean_rgb[3 * pixel + 1], P.mean_rgb[3 * pixel + 2]);
                } else {
                    mean = rgb(0, 0, 0);
                }
                sample = 0;
                st = ST_CAMERA;
                break;
            }
            case ST_CAMERA: {
                // optix_pathtracing_kernels.cu:43-55, 76-81.
                uint32_t img_w = static_cast<uint32_t>(P.width), img_h = static_cast<uint32_t>(P.height);
                if (kMayTrain && is_train) {
                    img_w = kCombo ? set_w(tset) : train_w;
                    img_h = kCombo ? set_h(tset) : train_h;
                }
                uint32_t px = pixel % img_w;
                uint32_t py = pixel / img_w;
                float ux = rng.uniform();
                float fx = (px + ux) / static_cast<float>(img_w);
                float uy = rng.uniform();
                float fy = (py + uy) / static_cast<float>(img_h);
                sqrt_spread = 0.0f;
                prev_vertex = kInvalidVertex;
                terminal_written = false;
                const float cam_vw = P.cam_aspect * cam_vh;
                const float sensor_area = cam_vw * cam_vh;
                origin = v3(P.cam_pos[0], P.cam_pos[1], P.cam_pos[2]);
                V3 local = normalize(v3(cam_vw * (-0.5f + fx), cam_vh * (0.5f - fy), -1));
                dir = normalize(mul(quat_to_m3(P.cam_quat[0], P.cam_quat[1], P.cam_quat[2], P.cam_quat[3]), local));
                float az = fabsf(local.z);
                dir_pdf = 1 / (az * az * az * sensor_area);
                float inv = 1.0f / dir_pdf;
                throughput = rgb(1, 1, 1) * inv;
                init_importance = luminance(throughput);
                contribution = rgb(0, 0, 0);
                path_length = 0;
                end_code = 0;
                rec_primary = rec_shadow = 0;
                st = ST_SEGMENT;
                break;
            }
            case ST_SEGMENT: {
                ++path_length;
                ++n_vertices;
                if (path_length > kHardVertexCap) {
                    end_code = END_MAX_BOUNCES;
                    st = ST_END_SAMPLE;
                    break;
                }
                // optix_pathtracing_kernels.cu:84-96: the closest triangle bounds the segment.
                float seg_max = 1e10f;
                bool in_volume = true;
                if constexpr (kSurfaces) {
                    bool overflow = false;
                    const SurfHit h = bvh_closest(P.surf, origin, dir, 0.0f, 1e10f, &overflow);
                    if (overflow) err |= VPT_DEVERR_BVH_STACK;
                    hit_tri = h.tri;
                    hit_b1 = h.b1;
                    hit_b2 = h.b2;
                    if (h.tri != ~0u) seg_max = h.t;
                    in_volume = P.volume_enabled != 0;
                }
                float a, b;
                if (in_volume && clip_ray(bmin, bmax, origin, dir, 0.0f, seg_max, &a, &b)) {
                    shadow = false;
                    t = fmaxf(0.0f, a);
                    t1 = b;
                    seg_steps = 0;
                    if constexpr (kGridMajorant) {
                        dda_init(g, origin, dir, t, &dda);
                        texit = fminf(fminf(dda.tnext[0], dda.tnext[1]), fminf(dda.tnext[2], t1));
                        maj = P.density_coeff * cell_maj(maj_grid, g, dda);
                    } else {
                        maj = global_maj;
                    }
                    st = ST_STEP;
                } else {
                    st = (kSurfaces && hit_tri != ~0u) ? ST_SURFACE : ST_ESCAPE;
                }
                break;
            }
            case ST_STEP: {
                const V3 seg_dir = shadow ? -light_dir : dir;
                constexpr int kCells = kMode == kModePlain ? (kSurfaces ? kSurfCellStepsPerPass : kCellStepsPerPass)
                                                           : kNrcCellStepsPerPass;
                const int r = track_pass<kGridMajorant, kCells>(g, maj_grid, P.density_coeff, t1, seg_dir, rng, t, texit,
                                                                maj, dda, n_cells);
                if (r == PASS_LOOKUP) {
                    V3 seg_eye;
                    if constexpr (kSurfaces)
                        seg_eye = shadow ? shadow_eye : origin;
                    else
                        seg_eye = shadow ? origin + trace_len * light_dir : origin;
                    lookup_pos = seg_eye + seg_dir * t;
                    need_lookup = true;
                } else if (r == PASS_END) {
                    st = shadow ? ST_NEE_DONE : ((kSurfaces && hit_tri != ~0u) ? ST_SURFACE : ST_ESCAPE);
                } else {
                    yield = true;  // let the warp's lookups run before crossing more cells
                }
                break;
            }
            case ST_ESCAPE: {
                // optix_pathtracing_kernels.cu:130-174.
                if (P.env_enabled) {
                    float hyp_pdf;
                    RGB radiance = env_evaluate<kNrc>(P.env, dir, &hyp_pdf);
                    float mis = 1.0f;
                    if (path_length > 1) {
                        float sel = P.sun.enabled ? (1.0f - P.sun.select_prob) : 1.0f;
                        // :140-142: with emitting triangles the environment is picked with
                        // probToSampleEnvLight.
                        if constexpr (kSurfaces) {
                            if (P.surf.inst_integral > 0.0f) sel = P.sun.enabled ? kProbEnvLight * sel : kProbEnvLight;
                        }
                        float light_pdf = sel * hyp_pdf;
                        float bsdf_pdf = dir_pdf;
                        mis = (bsdf_pdf * bsdf_pdf) / ((bsdf_pdf * bsdf_pdf) + (light_pdf * light_pdf));
                    }
                    const RGB implicit = radiance * mis;
                    if (!(kMayTrain && is_train)) contribution = contribution + throughput * implicit;
                    if (kMayTrain && is_train) {
                        // :148-152: the environment hit completes the previous vertex's target.
                        if (prev_vertex != kInvalidVertex) {
                            // The previous vertex's local throughput, as this lane recorded it.
                            const TrainVertexInfo& pv = tr_vertex()[prev_vertex];
                            float* tg = tr_target0() + 3 * static_cast<size_t>(prev_vertex);
                            RGB add = rgb(pv.local_tp[0], pv.local_tp[1], pv.local_tp[2]) * implicit;
                            tg[0] += add.r;
                            tg[1] += add.g;
                            tg[2] += add.b;
                        }
                    }
                }
                end_code = END_ESCAPE;
                st = ST_END_SAMPLE;
                break;
            }
            case ST_VERTEX: {
                // In-medium vertex (:176-182), Russian roulette (:254-268, 332), NEE set-up
                // (renderer_kernel_common.h:297-358).
                const V3 seg_origin = origin;
                origin = origin + t * dir;
                if constexpr (kNrc) {
                    // optix_pathtracing_kernels.cu:200-210: path spread (|cos| = 1 in a medium).
                    V3 dv = seg_origin - origin;
                    float dist2 = dv.x * dv.x + dv.y * dv.y + dv.z * dv.z;
                    if (path_length == 1)
                        primary_spread = dist2 / (4 * kPi * 1.0f);
                    else
                        sqrt_spread += sqrtf(dist2 / (dir_pdf * 1.0f));
                }
                float continue_prob = 1.0f;
                bool rr_kill = false;
                // Training suffixes apply Russian roulette from the third vertex (:256-257).
                const int32_t rr_from = (kMayTrain && is_train) ? max(P.rr_start, 3) : P.rr_start;
                if (static_cast<int32_t>(path_length) >= rr_from) {
                    continue_prob = fminf(luminance(throughput) / init_importance, 1.0f);
                    if (rng.uniform() >= continue_prob) rr_kill = true;
                }
                if constexpr (!kNrc) {
                    if (rr_kill) {
                        end_code = END_RR;
                        st = ST_END_SAMPLE;
                        break;
                    }
                } else {
                    // :282-330: the path ends with a cache query on Russian roulette or once its
                    // spread exceeds the primary footprint (twice that for biased training suffixes).
                    bool ends_with_cache = rr_kill;
                    const float spread2 = sqrt_spread * sqrt_spread;
                    if (kMayTrain && is_train) {
                        if (!unbiased) ends_with_cache |= spread2 > train_term_factor * primary_spread;
                    } else {
                        ends_with_cache |= spread2 > term_factor * primary_spread;
                    }
                    if (ends_with_cache) {
                        const float rough = P.nrc_density_query && P.density_coeff > 0 ? last_density / P.density_coeff : 0.0f;
                        float* qdst = (kMayTrain && is_train) ? tr_end_query() : P.nrc.infer_query;
                        write_query(qdst + kQueryFloats * static_cast<size_t>(slot), origin, -dir, rough, P.albedo, wmin,
                                    wmax);
                        end_with_query();
                        break;
                    }
                }
                throughput = rdiv(throughput, continue_prob);
                if constexpr (kSurfaces) {
                    at_surface = false;
                    st = ST_NEE_SETUP;
                    break;
                }

                float u_light = rng.uniform();
                float u0 = rng.uniform();
                float u1 = rng.uniform();
                pick_sun = false;
                float light_prob = 1.0f;
                bool have_light = true;
                if (P.sun.enabled && P.env_enabled) {
                    if (u_light < P.sun.select_prob) {
                        pick_sun = true;
                        light_prob = P.sun.select_prob;
                    } else {
                        light_prob = 1.0f - P.sun.select_prob;
                    }
                } else if (P.sun.enabled) {
                    pick_sun = true;
                } else if (!P.env_enabled) {
                    have_light = false;
                }
                vis = 0.0f;
                if (have_light) {
                    if (pick_sun) {
                        light_dir = v3(P.sun.dir[0], P.sun.dir[1], P.sun.dir[2]);
                        emittance = rgb(P.sun.irradiance[0], P.sun.irradiance[1], P.sun.irradiance[2]);
                        area_pdf = light_prob;
                    } else {
                        float pdf;
                        RGB radiance = env_sample(P.env, u0, u1, &light_dir, &pdf);
                        emittance = kPi * radiance;
                        area_pdf = pdf;
                        if (area_pdf == 0.0f) have_light = false;
                        area_pdf *= light_prob;
                    }
                }
                if (have_light) {
                    V3 sdir = -light_dir;
                    float lp_cos = dot(sdir, -light_dir);
                    if (lp_cos <= 0.0f) have_light = false;
                }
                if (!have_light) {
                    st = ST_NEE_DONE;  // vis = 0: no contribution
                    break;
                }
                vis = 1.0f;
                const V3 seg_dir = -light_dir;
                const V3 seg_eye = origin + trace_len * light_dir;
                float a, b;
                if (clip_ray(bmin, bmax, seg_eye, seg_dir, 0.0f, trace_len, &a, &b)) {
                    shadow = true;
                    t = fmaxf(0.0f, a);
                    t1 = b;
                    seg_steps = 0;
                    if constexpr (kGridMajorant) {
                        dda_init(g, seg_eye, seg_dir, t, &dda);
                        texit = fminf(fminf(dda.tnext[0], dda.tnext[1]), fminf(dda.tnext[2], t1));
                        maj = P.density_coeff * cell_maj(maj_grid, g, dda);
                    } else {
                        maj = global_maj;
                    }
                    st = ST_STEP;
                } else {
                    st = ST_NEE_DONE;
                }
                break;
            }
            case ST_SURFACE: {
                if constexpr (kSurfaces) {
                    // A triangle hit (optix_pathtracing_kernels.cu:176-195): the surface point,
                    // its emission weighted against area-light sampling (:216-239), Russian
                    // roulette (:254-268), NEE set-up.
                    const SurfPoint sp = surface_point(P.surf, hit_tri, hit_b1, hit_b2, P.env_enabled != 0);
                    const V3 ray_origin = origin;
                    origin = sp.pos;
                    const V3 vout_local = to_local(sp.sf, -dir);
                    const SurfMaterial& mt = P.surf.mats[sp.material];
                    if constexpr (kNrc) {
                        // :200-210: path spread, |cos| against the geometric normal.
                        const V3 dv = ray_origin - origin;
                        const float dist2 = dv.x * dv.x + dv.y * dv.y + dv.z * dv.z;
                        const float abs_dot = fabsf(dot(dir, sp.gn));
                        if (path_length == 1)
                            primary_spread = dist2 / (4 * kPi * abs_dot);
                        else
                            sqrt_spread += sqrtf(dist2 / (dir_pdf * abs_dot));
                    }
                    if (vout_local.z > 0 && mt.emissive) {
                        const RGB em = rgb(mt.emittance[0], mt.emittance[1], mt.emittance[2]);
                        float mis = 1.0f;
                        if (path_length > 1) {
                            const V3 dv = ray_origin - origin;
                            const float dist2 = dot(dv, dv);
                            const float light_pdf = sp.hyp_area_pdf * dist2 / vout_local.z;
                            const float bsdf_pdf = dir_pdf;
                            mis = (bsdf_pdf * bsdf_pdf) / ((bsdf_pdf * bsdf_pdf) + (light_pdf * light_pdf));
                        }
                        const RGB implicit = em * (mis / kPi);
                        if (!(kMayTrain && is_train)) contribution = contribution + throughput * implicit;
                        if (kMayTrain && is_train && prev_vertex != kInvalidVertex) {
                            // :231-237: the emission completes the previous vertex's target.
                            const TrainVertexInfo& pv = tr_vertex()[prev_vertex];
                            float* tg = tr_target0() + 3 * static_cast<size_t>(prev_vertex);
                            const RGB add = rgb(pv.local_tp[0], pv.local_tp[1], pv.local_tp[2]) * implicit;
                            tg[0] += add.r;
                            tg[1] += add.g;
                            tg[2] += add.b;
                        }
                    }
                    float continue_prob = 1.0f;
                    bool rr_kill = false;
                    const int32_t rr_from = (kMayTrain && is_train) ? max(P.rr_start, 3) : P.rr_start;
                    if (static_cast<int32_t>(path_length) >= rr_from) {
                        continue_prob = fminf(luminance(throughput) / init_importance, 1.0f);
                        if (rng.uniform() >= continue_prob) rr_kill = true;
                    }
                    if constexpr (!kNrc) {
                        if (rr_kill) {
                            end_code = END_RR;
                            st = ST_END_SAMPLE;
                            break;
                        }
                    } else {
                        // :282-330 at a surface: the query holds the shading normal and the
                        // material's reflectances and roughness.
                        bool ends_with_cache = rr_kill;
                        const float spread2 = sqrt_spread * sqrt_spread;
                        if (kMayTrain && is_train) {
                            if (!unbiased) ends_with_cache |= spread2 > train_term_factor * primary_spread;
                        } else {
                            ends_with_cache |= spread2 > term_factor * primary_spread;
                        }
                        if (ends_with_cache) {
                            float* qdst = (kMayTrain && is_train) ? tr_end_query() : P.nrc.infer_query;
                            write_query_surface(qdst + kQueryFloats * static_cast<size_t>(slot), origin, sp.sf.n, -dir,
                                                mt, wmin, wmax);
                            end_with_query();
                            break;
                        }
                    }
                    throughput = rdiv(throughput, continue_prob);
                    at_surface = true;
                    st = ST_NEE_SETUP;
                } else {
                    st = ST_ESCAPE;
                }
                break;
            }
            case ST_NEE_SETUP: {
                // One call site for medium and surface vertices keeps the kernel's code small
                // (the surface passes are bound by instruction fetch otherwise).
                if constexpr (kSurfaces) surf_nee_setup();
                break;
            }
            case ST_NEE_DONE: {
                if constexpr (kSurfaces) {
                    if (at_surface) {
                        // renderer_kernel_common.h:385-402 with the surface's BSDF, then BSDF
                        // sampling and the offset origin of the next ray
                        // (optix_pathtracing_kernels.cu:340-356).
                        const SurfPoint sp = surface_point(P.surf, hit_tri, hit_b1, hit_b2, P.env_enabled != 0);
                        const SurfMaterial& mt = P.surf.mats[sp.material];
                        const Bsdf f = make_bsdf(mt);
                        const V3 q = to_local(sp.sf, -dir);
                        RGB nee_s = rgb(0, 0, 0);
                        if (vis > 0.0f) {
                            const V3 sdir = -light_dir;
                            const V3 vin = to_local(sp.sf, -sdir);
                            float bpdf0;
                            const RGB fs = bsdf_eval_pdf(f, q, vin, &bpdf0);
                            const float sp_cos = fabsf(dot(sdir, sp.gn));
                            RGB nee;
                            if (pick_sun) {
                                nee = fs * emittance * (vis * sp_cos / area_pdf);
                            } else {
                                float bpdf = bpdf0 * nee_lp_cos / nee_dist2;
                                if (!isfinite(bpdf)) bpdf = 0.0f;
                                const float light_pdf = area_pdf;
                                const float mis = (light_pdf * light_pdf) / ((bpdf * bpdf) + (light_pdf * light_pdf));
                                const RGB le = rdiv(emittance, kPi);
                                const float gterm = nee_lp_cos * sp_cos / nee_dist2;
                                nee = fs * le * (vis * mis * gterm / area_pdf);
                            }
                            if (!(kMayTrain && is_train)) contribution = contribution + throughput * nee;
                            nee_s = nee;
                        }
                        if (P.max_bounces > 0 && static_cast<int32_t>(path_length) >= P.max_bounces) {
                            end_code = END_MAX_BOUNCES;
                            st = ST_END_SAMPLE;
                            break;
                        }
                        const float u0 = rng.uniform();
                        const float u1 = rng.uniform();
                        V3 local;
                        float pdf;
                        const RGB fs = bsdf_sample(f, q, u0, u1, &local, &pdf);
                        if (pdf == 0.0f) {
                            end_code = END_PDF_ZERO;
                            st = ST_END_SAMPLE;
                            break;
                        }
                        const V3 v_out = -dir;
                        dir = from_local(sp.sf, local);
                        const float dot_sgn = dot(dir, sp.gn);
                        const RGB local_tp = fs * (fabsf(dot_sgn) / pdf);
                        throughput = throughput * local_tp;
                        origin = offset_ray_origin(sp.pos, (dot_sgn > 0.0f ? 1.0f : -1.0f) * sp.gn);
                        dir_pdf = pdf;
                        at_surface = false;
                        st = ST_SEGMENT;
                        if (kMayTrain && is_train) {
                            // :358-409 at a surface vertex: the query at the surface point (not the
                            // offset origin), the BSDF's local throughput, the NEE target.
                            const uint32_t idx = atomicAdd(tr_counters() + tr_buf(), 1u);
                            if (idx < kTrainBufferSize) {
                                write_query_surface(tr_query0() + kQueryFloats * static_cast<size_t>(idx), sp.pos, sp.sf.n,
                                                    v_out, mt, wmin, wmax);
                                TrainVertexInfo vi;
                                vi.local_tp[0] = local_tp.r;
                                vi.local_tp[1] = local_tp.g;
                                vi.local_tp[2] = local_tp.b;
                                vi.bits = (prev_vertex & kInvalidVertex) | ((path_length & 0xFFu) << 22) |
                                          ((unbiased ? 1u : 0u) << 30);
                                tr_vertex()[idx] = vi;
                                float* tg = tr_target0() + 3 * static_cast<size_t>(idx);
                                tg[0] = nee_s.r;
                                tg[1] = nee_s.g;
                                tg[2] = nee_s.b;
                                prev_vertex = idx;
                            } else {
                                write_query_surface(tr_end_query() + kQueryFloats * static_cast<size_t>(slot), sp.pos,
                                                    sp.sf.n, v_out, mt, wmin, wmax);
                                tr_suffix()[slot] = pack_suffix(prev_vertex, 1, path_length, unbiased ? 1 : 0);
                                terminal_written = true;
                                err |= VPT_DEVERR_TRAIN_FULL;
                                end_code = END_TRAIN_FULL;
                                st = ST_END_SAMPLE;
                            }
                        }
                        break;
                    }
                }
                // renderer_kernel_common.h:385-402, then phase sampling (:341-356).
                nee_value = rgb(0, 0, 0);
                if (vis > 0.0f) {
                    V3 sdir = -light_dir;
                    Frame fr = make_frame(-dir);
                    V3 v_in_local = to_local(fr, -sdir);
                    float pf = phase_pdf(P.phase_kind, P.phase_param, v_in_local);
                    RGB fs = rgb(P.albedo, P.albedo, P.albedo) * pf;
                    RGB nee;
                    if (pick_sun) {
                        nee = fs * emittance * (vis / area_pdf);
                    } else {
                        // Surface scenes keep the light-side cosine over the distance and the
                        // squared distance of an area-light sample (1 for the environment).
                        float lp_cos = kSurfaces ? nee_lp_cos : dot(sdir, -light_dir);
                        const float dist2 = kSurfaces ? nee_dist2 : 1.0f;
                        float bsdf_pdf = pf * lp_cos / dist2;
                        if (!isfinite(bsdf_pdf)) bsdf_pdf = 0.0f;
                        float light_pdf = area_pdf;
                        float mis = (light_pdf * light_pdf) / ((bsdf_pdf * bsdf_pdf) + (light_pdf * light_pdf));
                        RGB le = rdiv(emittance, kPi);
                        float gterm = lp_cos * 1.0f / dist2;
                        nee = fs * le * (vis * mis * gterm / area_pdf);
                    }
                    if (!(kMayTrain && is_train)) contribution = contribution + throughput * nee;
                    nee_value = nee;
                }
                if (P.max_bounces > 0 && static_cast<int32_t>(path_length) >= P.max_bounces) {
                    end_code = END_MAX_BOUNCES;
                    st = ST_END_SAMPLE;
                    break;
                }
                Frame fr = make_frame(-dir);
                float u0 = rng.uniform();
                float u1 = rng.uniform();
                V3 local;
                float pdf = phase_sample(P.phase_kind, P.phase_param, u0, u1, &local);
                if (pdf == 0.0f) {
                    end_code = END_PDF_ZERO;
                    st = ST_END_SAMPLE;
                    break;
                }
                RGB fs = rgb(P.albedo, P.albedo, P.albedo) * pdf;
                const V3 v_out = -dir;
                dir = from_local(fr, local);
                RGB local_tp = fs * (fabsf(1.0f) / pdf);
                throughput = throughput * local_tp;
                dir_pdf = pdf;
                if (kMayTrain && is_train) {
                    // :358-409: record the training vertex (query, local throughput, link to the
                    // previous vertex, target initialised with the NEE estimate); a full buffer
                    // ends the suffix with a cache query.
                    const uint32_t idx = atomicAdd(tr_counters() + tr_buf(), 1u);
                    const float rough = P.nrc_density_query && P.density_coeff > 0 ? last_density / P.density_coeff : 0.0f;
                    if (idx < kTrainBufferSize) {
                        write_query(tr_query0() + kQueryFloats * static_cast<size_t>(idx), origin, v_out, rough,
                                    P.albedo, wmin, wmax);
                        TrainVertexInfo vi;
                        vi.local_tp[0] = local_tp.r;
                        vi.local_tp[1] = local_tp.g;
                        vi.local_tp[2] = local_tp.b;
                        vi.bits = (prev_vertex & kInvalidVertex) | ((path_length & 0xFFu) << 22) | ((unbiased ? 1u : 0u) << 30);
                        tr_vertex()[idx] = vi;
                        float* tg = tr_target0() + 3 * static_cast<size_t>(idx);
                        tg[0] = nee_value.r;
                        tg[1] = nee_value.g;
                        tg[2] = nee_value.b;
                        prev_vertex = idx;
                    } else {
                        write_query(tr_end_query() + kQueryFloats * static_cast<size_t>(slot), origin, v_out,
                                    rough, P.albedo, wmin, wmax);
                        tr_suffix()[slot] = pack_suffix(prev_vertex, 1, path_length, unbiased ? 1 : 0);
                        terminal_written = true;
                        err |= VPT_DEVERR_TRAIN_FULL;
                        end_code = END_TRAIN_FULL;
                        st = ST_END_SAMPLE;
                        break;
                    }
                }
                st = ST_SEGMENT;
                break;
            }
            case ST_END_SAMPLE: {
                // optix_pathtracing_kernels.cu:413-432 (non-finite samples are dropped).
                ++n_samples;
                if constexpr (kNrc) {
                    if (kMayTrain && is_train) {
                        if (!terminal_written)
                            tr_suffix()[slot] = pack_suffix(prev_vertex, 0, path_length, unbiased ? 1 : 0);
                    } else {
                        if (!terminal_written) {
                            TerminalInfo ti;
                            ti.tp[0] = throughput.r;
                            ti.tp[1] = throughput.g;
                            ti.tp[2] = throughput.b;
                            ti.bits = (path_length & 0xFFu) << 1;
                            P.nrc.infer_terminal[slot] = ti;
                        }
                        RGB c = contribution;
                        if (!all_nonneg_finite(c)) {
                            err |= VPT_DEVERR_NONFINITE;
                            c = rgb(0, 0, 0);
                        }
                        float* fc = P.nrc.frame_contribution + 3 * static_cast<size_t>(slot);
                        fc[0] = c.r;
                        fc[1] = c.g;
                        fc[2] = c.b;
                    }
                    if ((kMayTrain && is_train) || !sample_parallel)
                        ((kCombo && is_train) ? P.train_sets[tset].rng : P.rng)[rng_index] = rng.state;
                    st = ST_FETCH;
                    break;
                }
                if constexpr (kLog) {
                    uint4 rec = make_uint4(path_length, rec_primary, rec_shadow, end_code);
                    reinterpret_cast<uint4*>(P.dlog)[static_cast<uint64_t>(pixel) * P.spp + sample] = rec;
                }
                if (sample_parallel) {
                    if (all_nonneg_finite(contribution)) {
                        atomicAdd(P.sum_rgb + 3 * pixel, static_cast<double>(contribution.r));
                        atomicAdd(P.sum_rgb + 3 * pixel + 1, static_cast<double>(contribution.g));
                        atomicAdd(P.sum_rgb + 3 * pixel + 2, static_cast<double>(contribution.b));
                    } else {
                        err |= VPT_DEVERR_NONFINITE;
                    }
                    st = ST_FETCH;
                    break;
                }
                if (all_nonneg_finite(contribution)) {
                    sum_r += contribution.r;
                    sum_g += contribution.g;
                    sum_b += contribution.b;
                    uint32_t n = P.accum_base + sample;
                    RGB prev = n > 0 ? mean : rgb(0, 0, 0);
                    float w = 1.0f / (n + 1);
                    mean = (1 - w) * prev + w * contribution;
                } else {
                    err |= VPT_DEVERR_NONFINITE;
                }
                ++sample;
                if (sample < P.spp) {
                    st = ST_CAMERA;
                } else {
                    P.rng[pixel] = rng.state;
                    P.sum_rgb[3 * pixel] += sum_r;
                    P.sum_rgb[3 * pixel + 1] += sum_g;
                    P.sum_rgb[3 * pixel + 2] += sum_b;
                    P.mean_rgb[3 * pixel] = mean.r;
                    P.mean_rgb[3 * pixel + 1] = mean.g;
                    P.mean_rgb[3 * pixel + 2] = mean.b;
                    st = ST_FETCH;
                }
                break;
            }
            default:
                st = ST_DONE;
                break;
            }
        }

        if (event_phase || !__any_sync(0xffffffffu, need_lookup)) continue;

        // ---------------------------------------------------------------- converged lookups
        float density = 0.0f;
        if constexpr (kStage) {
            density = P.density_coeff * sample_trilinear_staged(g, need_lookup, world_to_index(g, lookup_pos), leaf_cache,
                                                                 stage, P.leaf_stage_min, stage_timed_out);
        } else {
            if (need_lookup) density = P.density_coeff * sample_trilinear(g, world_to_index(g, lookup_pos), leaf_cache);
        }

        // Outcome of one lookup at the lane's current tentative collision (majorant `maj`).
        auto resolve = [&](float dens) {
            ++n_lookups;
            ++seg_steps;
            if (shadow) {
                ++rec_shadow;
                vis *= (1 - dens / maj);
                // Russian roulette on the remaining visibility (configuration mode). Training
                // suffixes keep plain ratio tracking: their NEE estimates are the cache's targets.
                const float rr_thr = (kMayTrain && is_train) ? 0.0f : P.shadow_rr;
                if (vis < rr_thr) {
                    const float q = vis / rr_thr;
                    if (rng.uniform() >= q) {
                        vis = 0.0f;
                        st = ST_NEE_DONE;
                    } else {
                        vis = rr_thr;
                    }
                }
            } else {
                ++rec_primary;
                if (rng.uniform() < dens / maj) {
                    st = ST_VERTEX;
                    last_density = dens;
                }
            }
            if (st == ST_STEP && seg_steps >= step_cap) {
                err |= VPT_DEVERR_STEP_CAP;
                end_code = END_STEP_CAP;
                st = ST_END_SAMPLE;
            }
        };
        if (need_lookup) resolve(density);
    }

    if constexpr (kStage) {
        if (stage_timed_out) {
            // A copy that did not complete may still land in this warp's buffer: wait for it
            // (again bounded) before the CTA's shared memory is released.
            err |= VPT_DEVERR_STAGE_TIMEOUT;
            stage_wait(stage.bar, stage.phase ^ 1u);
        }
    }

    // warp-reduce the work counters
    unsigned long long c_lookups = n_lookups, c_vertices = n_vertices, c_samples = n_samples, c_cells = n_cells;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c_lookups += __shfl_down_sync(0xffffffffu, c_lookups, o);
        c_vertices += __shfl_down_sync(0xffffffffu, c_vertices, o);
        c_samples += __shfl_down_sync(0xffffffffu, c_samples, o);
        c_cells += __shfl_down_sync(0xffffffffu, c_cells, o);
    }
    err = __reduce_or_sync(0xffffffffu, err);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(P.counters + 0, c_lookups);
        atomicAdd(P.counters + 1, c_vertices);
        atomicAdd(P.counters + 2, c_samples);
        atomicAdd(P.counters + 3, c_cells);
        if (err) atomicOr(P.error_flags, err);
    }
}

// Mean image of the sample-parallel mode: FP64 sums over the samples accumulated so far.
__global__ void finalize_mean_kernel(const double* __restrict__ sum, float* __restrict__ mean, uint32_t n,
                                     double inv_samples) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        mean[i] = static_cast<float>(sum[i] * inv_samples);
}

// Majorant grid of 2^shift-voxel cells from the 8^3-voxel cells (max-pooling by 2^(shift-3)).
__global__ void pool_majorants_kernel(const float* __restrict__ fine, int lx, int ly, int lz, float* __restrict__ out,
                                      int mx, int my, int mz, int factor) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mx * my * mz) return;
    int cz = i % mz, cy = (i / mz) % my, cx = i / (mz * my);
    float m = 0.0f;
    for (int x = cx * factor; x < min((cx + 1) * factor, lx); ++x)
        for (int y = cy * factor; y < min((cy + 1) * factor, ly); ++y)
            for (int z = cz * factor; z < min((cz + 1) * factor, lz); ++z)
                m = fmaxf(m, fine[(static_cast<int64_t>(x) * ly + y) * lz + z]);
    out[i] = m;
}

// Entry i: LCG jump (multiplier, increment) advancing a pixel's seed state by (first + i) * 2^40
// draws, the start of that sample's stream (O(log) jump-ahead, Brown 1994).
__global__ void sample_jump_table_kernel(ulonglong2* out, uint32_t first, uint32_t count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    uint64_t delta = static_cast<uint64_t>(first + i) << kSampleStreamShift;
    uint64_t cur_mult = 6364136223846793005ULL, cur_plus = 1ULL, acc_mult = 1ULL, acc_plus = 0ULL;
    while (delta > 0) {
        if (delta & 1ULL) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1ULL) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1;
    }
    out[i] = make_ulonglong2(acc_mult, acc_plus);
}

// As sample_jump_table_kernel, with the first sample index read from the context's device
// frame counters (so that a launch captured in a CUDA graph continues the streams on replay).
__global__ void sample_jump_table_dev_kernel(ulonglong2* out, const uint32_t* __restrict__ frame, uint32_t count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    uint64_t delta = static_cast<uint64_t>(frame[0] + i) << kSampleStreamShift;
    uint64_t cur_mult = 6364136223846793005ULL, cur_plus = 1ULL, acc_mult = 1ULL, acc_plus = 0ULL;
    while (delta > 0) {
        if (delta & 1ULL) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1ULL) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1;
    }
    out[i] = make_ulonglong2(acc_mult, acc_plus);
}

// mean = sum / (accumulated samples + spp), the count read from the device frame counters.
__global__ void finalize_mean_dev_kernel(const double* __restrict__ sum, float* __restrict__ mean, uint32_t n,
                                         const uint32_t* __restrict__ frame, uint32_t spp) {
    const double inv = 1.0 / (static_cast<double>(frame[1]) + spp);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        mean[i] = static_cast<float>(sum[i] * inv);
}

// frame[0] += add_stream; frame[1] = set ? value : frame[1] + value.
__global__ void frame_update_kernel(uint32_t* frame, uint32_t add_stream, int set_accum, uint32_t value) {
    frame[0] += add_stream;
    frame[1] = set_accum ? value : frame[1] + value;
}

}  // namespace

void launch_sample_jump_table_dev(ulonglong2* out, const uint32_t* frame, uint32_t count, cudaStream_t s) {
    sample_jump_table_dev_kernel<<<(count + 127) / 128, 128, 0, s>>>(out, frame, count);
}
void launch_finalize_mean_dev(const double* sum, float* mean, uint32_t n_values, const uint32_t* frame, uint32_t spp,
                              cudaStream_t s) {
    finalize_mean_dev_kernel<<<(n_values + 255) / 256, 256, 0, s>>>(sum, mean, n_values, frame, spp);
}
void launch_frame_update(uint32_t* frame, uint32_t add_stream, bool set_accum, uint32_t value, cudaStream_t s) {
    frame_update_kernel<<<1, 1, 0, s>>>(frame, add_stream, set_accum ? 1 : 0, value);
}

void launch_sample_jump_table(ulonglong2* out, uint32_t first, uint32_t count, cudaStream_t s) {
    sample_jump_table_kernel<<<(count + 127) / 128, 128, 0, s>>>(out, first, count);
}

void launch_finalize_mean(const double* sum, float* mean, uint32_t n_values, uint32_t samples, cudaStream_t s) {
    finalize_mean_kernel<<<(n_values + 255) / 256, 256, 0, s>>>(sum, mean, n_values, 1.0 / samples);
}

void pool_majorants(const float* fine, int lx, int ly, int lz, float* out, int mx, int my, int mz, int factor,
                    cudaStream_t s) {
    int n = mx * my * mz;
    pool_majorants_kernel<<<(n + 255) / 256, 256, 0, s>>>(fine, lx, ly, lz, out, mx, my, mz, factor);
}

size_t plain_smem_bytes(size_t maj_bytes, bool leaf_stage, int threads) {
    if (!leaf_stage) return maj_bytes;
    const size_t warps = static_cast<size_t>(threads) / 32;
    return (maj_bytes + 127) / 128 * 128 + warps * (kLeafBytes + sizeof(uint64_t));
}

// Logged launches (decision records for the parity tests) follow the stream layout at run time;
// the production launches use a kernel compiled for their layout. Leaf staging exists for the
// majorant-grid tracker on sample-parallel streams and for its logged form.
const void* plain_kernel_ptr(bool grid_majorant, bool logged, bool sample_parallel, bool leaf_stage) {
    if (leaf_stage && grid_majorant)
        return logged ? reinterpret_cast<const void*>(plain_trace_kernel<true, true, kModePlain, kStreamsRuntime, true>)
                      : reinterpret_cast<const void*>(
                            plain_trace_kernel<true, false, kModePlain, kStreamsSampleParallel, true>);
    if (logged) return grid_majorant ? reinterpret_cast<const void*>(plain_trace_kernel<true, true, kModePlain>)
                                     : reinterpret_cast<const void*>(plain_trace_kernel<false, true, kModePlain>);
    if (sample_parallel)
        return grid_majorant
                   ? reinterpret_cast<const void*>(plain_trace_kernel<true, false, kModePlain, kStreamsSampleParallel>)
                   : reinterpret_cast<const void*>(plain_trace_kernel<false, false, kModePlain, kStreamsSampleParallel>);
    return grid_majorant ? reinterpret_cast<const void*>(plain_trace_kernel<true, false, kModePlain, kStreamsPerPixel>)
                         : reinterpret_cast<const void*>(plain_trace_kernel<false, false, kModePlain, kStreamsPerPixel>);
}

void launch_plain(const TraceParams& p, bool grid_majorant, int grid_ctas, int threads, size_t smem, cudaStream_t s) {
    dim3 grid(grid_ctas), block(threads);
    const size_t sm = grid_majorant ? smem : 0;
    if (p.leaf_stage_min > 0 && grid_majorant && (p.dlog || p.stream_mode == 1)) {
        if (p.dlog)
            plain_trace_kernel<true, true, kModePlain, kStreamsRuntime, true><<<grid, block, sm, s>>>(p);
        else
            plain_trace_kernel<true, false, kModePlain, kStreamsSampleParallel, true><<<grid, block, sm, s>>>(p);
    } else if (p.dlog) {
        if (grid_majorant)
            plain_trace_kernel<true, true, kModePlain><<<grid, block, sm, s>>>(p);
        else
            plain_trace_kernel<false, true, kModePlain><<<grid, block, sm, s>>>(p);
    } else if (p.stream_mode == 1) {
        if (grid_majorant)
            plain_trace_kernel<true, false, kModePlain, kStreamsSampleParallel><<<grid, block, sm, s>>>(p);
        else
            plain_trace_kernel<false, false, kModePlain, kStreamsSampleParallel><<<grid, block, sm, s>>>(p);
    } else {
        if (grid_majorant)
            plain_trace_kernel<true, false, kModePlain, kStreamsPerPixel><<<grid, block, sm, s>>>(p);
        else
            plain_trace_kernel<false, false, kModePlain, kStreamsPerPixel><<<grid, block, sm, s>>>(p);
    }
}

template <bool kGridMajorant>
static const void* surface_kernel_for(bool logged) {
    return logged ? reinterpret_cast<const void*>(
                        plain_trace_kernel<kGridMajorant, true, kModePlain, kStreamsRuntime, false, true>)
                  : reinterpret_cast<const void*>(
                        plain_trace_kernel<kGridMajorant, false, kModePlain, kStreamsRuntime, false, true>);
}

const void* surface_kernel_ptr(bool grid_majorant, bool logged) {
    return grid_majorant ? surface_kernel_for<true>(logged) : surface_kernel_for<false>(logged);
}

void launch_surface(const TraceParams& p, bool grid_majorant, int grid_ctas, int threads, size_t smem, cudaStream_t s) {
    const size_t sm = grid_majorant ? smem : 0;
    void* args[] = {const_cast<TraceParams*>(&p)};
    cudaLaunchKernel(surface_kernel_ptr(grid_majorant, p.dlog != nullptr), dim3(grid_ctas), dim3(threads), args, sm, s);
}

template <int kMode, bool kSurfaces>
static const void* nrc_kernel_for(bool grid_majorant) {
    return grid_majorant
               ? reinterpret_cast<const void*>(plain_trace_kernel<true, false, kMode, kStreamsRuntime, false, kSurfaces>)
               : reinterpret_cast<const void*>(plain_trace_kernel<false, false, kMode, kStreamsRuntime, false, kSurfaces>);
}

const void* nrc_kernel_ptr(int mode, bool grid_majorant, bool surfaces) {
    if (surfaces) {
        if (mode == kModeTrainNrc) return nrc_kernel_for<kModeTrainNrc, true>(grid_majorant);
        if (mode == kModeComboNrc) return nrc_kernel_for<kModeComboNrc, true>(grid_majorant);
        return nrc_kernel_for<kModeRenderNrc, true>(grid_majorant);
    }
    if (mode == kModeTrainNrc) return nrc_kernel_for<kModeTrainNrc, false>(grid_majorant);
    if (mode == kModeComboNrc) return nrc_kernel_for<kModeComboNrc, false>(grid_majorant);
    return nrc_kernel_for<kModeRenderNrc, false>(grid_majorant);
}

void launch_nrc_pass(const TraceParams& p, int mode, bool grid_majorant, bool surfaces, int grid_ctas, int threads,
                     size_t smem, cudaStream_t s) {
    const size_t sm = grid_majorant ? smem : 0;
    void* args[] = {const_cast<TraceParams*>(&p)};
    cudaLaunchKernel(nrc_kernel_ptr(mode, grid_majorant, surfaces), dim3(grid_ctas), dim3(threads), args, sm, s);
}

}  // namespace vpt
