/*
 * rtc8_vpt.h — C ABI of the GB300 volumetric path tracer (plain and NRC render paths).
 *
 * This surface replaces the reference renderer's per-frame launch entry points
 * (shocker-0x15/rtcamp8):
 *   - the OptiX ray-generation programs pathTrace / generateTrainingData / pathTraceWithNRC
 *     (renderer/gpu_kernels/optix_pathtracing_kernels.cu:438-448), launched by
 *     optixPipeline.launch(stream, plp, w, h, 1) (renderer/renderer_main.cpp:1575-1577,
 *     1622-1624, 1640-1642);
 *   - the CUDA kernels prepareNRC, propagateRadianceValues, shuffleTrainingData and
 *     accumulateInferredRadianceValues (renderer/gpu_kernels/nrc_set_up_kernels.cu:4, 46,
 *     88, 176), launched with block 32 (renderer/renderer_main.cpp:1564-1592, 1635-1636);
 *   - the launch-parameter block PipelineLaunchParameters (renderer/renderer_shared.h:113-172),
 *     which becomes the opaque VptContext plus the POD structs below.
 *
 * Conventions: every call returns VPT_OK (0) or a negative VPT_ERR_* code (no exceptions
 * cross the ABI); `stream` is a cudaStream_t passed as void* (NULL = legacy default stream);
 * launches are asynchronous on that stream; a context is not thread-safe (the reference
 * renderer drives its pipeline from one host thread, renderer_main.cpp:1453-1454).
 */
#ifndef RTC8_VPT_H
#define RTC8_VPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VPT_OK 0
#define VPT_ERR_INVALID_ARGUMENT (-1)
#define VPT_ERR_CUDA (-2)
#define VPT_ERR_NOT_READY (-3)
#define VPT_ERR_OUT_OF_MEMORY (-4)
#define VPT_ERR_DEVICE_FAULT_FLAG (-5)

/* Device-side error bits reported by vpt_get_device_errors(). */
#define VPT_DEVERR_STEP_CAP 0x1u      /* a tracking segment hit max_steps_per_segment */
#define VPT_DEVERR_NONFINITE 0x2u     /* a non-finite sample contribution was dropped */
#define VPT_DEVERR_TRAIN_FULL 0x4u    /* the training-vertex buffer overflowed */
#define VPT_DEVERR_STAGE_TIMEOUT 0x8u /* a leaf-staging copy did not complete in time (staging stopped) */
#define VPT_DEVERR_BVH_STACK 0x10u    /* a surface BVH traversal ran out of stack (nodes skipped) */

typedef struct VptContext VptContext;

/* renderer_shared.h:144-167 (PerFramePipelineLaunchParameters) restricted to volumes, plus the
 * path rules and light model of the GB300 configurations. */
typedef struct VptFrameParams {
    /* PerspectiveCamera (common/common_renderer_types.h:1019-1034) */
    float cam_aspect;
    float cam_fovy;              /* radians */
    float cam_position[3];
    float cam_orientation[4];    /* quaternion x, y, z, w */

    float density_coeff;         /* sigma_t scale: sigma_t(x) = density_coeff * grid(x) */
    float scattering_albedo;
    int32_t phase_kind;          /* 0 = Schlick (reference), 1 = Henyey-Greenstein */
    float phase_param;           /* Schlick k (scatteringForwardness) or HG g */
    float radiance_scale;        /* NRC target scale (renderer_shared.h:160); <= 0 = off */

    int32_t env_enabled;
    float env_power;             /* powerCoeff */
    float env_rotation;          /* radians */

    int32_t sun_enabled;
    float sun_direction[3];      /* unit vector towards the sun */
    float sun_irradiance[3];
    float sun_select_prob;

    int32_t max_bounces;         /* 0 = no cap (reference) */
    int32_t rr_start_vertex;     /* Russian roulette from this path length (reference: 1) */
    int32_t majorant_mode;       /* 0 = global majorant (reference), 1 = 8^3 majorant grid DDA */
    int32_t max_steps_per_segment;  /* safety cap on lookups per segment (0 = none) */
    /* 0 = reference streams: one PCG32 stream per pixel, samples drawn one after the other
     *     (renderer_main.cpp:86-93, optix_pathtracing_kernels.cu:38, 413); a launch traces a
     *     pixel's samples in order, so the per-pixel chain bounds the launch time.
     * 1 = sample-parallel streams: sample s of a pixel starts from the pixel's seed state advanced
     *     by s * 2^40 draws (PCG jump-ahead), so every (pixel, sample) is an independent work item;
     *     the per-pixel seed states are not modified by a launch. */
    int32_t rng_stream_mode;
    /* log2 of the majorant-grid cell size in voxels (>= 3; 3 = one cell per 8^3 leaf). Larger
     * cells mean fewer DDA steps per ray and looser majorants. */
    int32_t majorant_cell_log2;
    /* Russian roulette on the transmittance of NEE shadow rays (configuration mode; 0 = off, the
     * reference's plain ratio tracking): once a shadow ray's visibility drops below this
     * threshold it survives with probability vis / threshold and continues with visibility
     * = threshold (unbiased); the extra random number is drawn from the path's stream. The
     * radiance-cache training passes ignore it (their NEE estimates are training targets). */
    float shadow_rr_threshold;
} VptFrameParams;

/* ---- context ------------------------------------------------------------------------ */
int vpt_create(int32_t image_width, int32_t image_height, VptContext** out);
int vpt_destroy(VptContext* ctx);
const char* vpt_last_error(void);

/* Per-pixel PCG32 states from one std::mt19937_64(seed) stream in row-major order
 * (renderer_main.cpp:86-93 uses seed 591842031321323413). Resets the accumulation. */
int vpt_seed_rng(VptContext* ctx, uint64_t seed);
int vpt_set_rng_states(VptContext* ctx, const uint64_t* host_states);
int vpt_get_rng_states(VptContext* ctx, uint64_t* host_states);

/* ---- scene data --------------------------------------------------------------------- */
/* Density grid from a dense voxel array (x-major: index = (x*ny + y)*nz + z) given as a HOST
 * pointer (vpt_set_volume_dense) or a DEVICE pointer (vpt_set_volume_dense_device). The grid
 * is stored on the device as NanoVDB-style 8^3 leaves (values ordered x<<6|y<<3|z) reached
 * through a dense leaf table; all-zero leaves are not stored. World position of voxel index
 * (i,j,k) is origin + (i,j,k) * voxel_size; the clip box is [origin, origin + n * voxel_size].
 * Replaces Scene::allocateVolumeGrid (renderer/renderer_scene.cpp:491-537), including its
 * global majorant scan over [min, max) of the index box (:498-509). */
int vpt_set_volume_dense(VptContext* ctx, const float* host_voxels, int32_t nx, int32_t ny,
                         int32_t nz, float voxel_size, const float origin[3]);
int vpt_set_volume_dense_device(VptContext* ctx, const float* dev_voxels, int32_t nx, int32_t ny,
                                int32_t nz, float voxel_size, const float origin[3]);
/* Seeded fBm value-noise volume generated on the device (octaves, lacunarity, gain, base
 * frequency in lattice cells across the grid). Values are remapped so min..max -> [0,1];
 * with threshold > 0 they become max(0, (r - threshold) / (1 - threshold)). */
int vpt_generate_fbm_volume(VptContext* ctx, int32_t n, uint32_t seed, int32_t octaves,
                            float lacunarity, float gain, float base_frequency, float threshold,
                            float voxel_size, const float origin[3]);
/* Union of two such clouds (seeds seed_a and seed_b, each remapped and thresholded on its own):
 * voxel = max of the two. */
int vpt_generate_fbm_union(VptContext* ctx, int32_t n, uint32_t seed_a, uint32_t seed_b, int32_t octaves,
                           float lacunarity, float gain, float base_frequency, float threshold,
                           float voxel_size, const float origin[3]);
/* Copies the dense voxel values of the last generated/uploaded volume to the host (n^3 floats);
 * only valid until the next volume call. */
int vpt_download_volume_dense(VptContext* ctx, float* host_voxels);
/* Grid statistics: active leaves, total leaves, global majorant, device bytes of the grid. */
int vpt_get_volume_info(VptContext* ctx, int64_t* active_leaves, int64_t* total_leaves,
                        float* global_majorant, int64_t* grid_bytes);
/* Per-cell majorants (one per 8^3 leaf cell, max over the cell's voxels plus a one-voxel
 * apron on every side) as a host copy of cx*cy*cz floats. */
int vpt_download_cell_majorants(VptContext* ctx, float* host_cells);

/* ---- NanoVDB grids ------------------------------------------------------------------- */
/* Description of one NanoVDB grid (format version 32.x). Filled from a file's metadata record
 * by vpt_nvdb_file_info (io::GridMetaData, ext/nanovdb/nanovdb/util/IO.h:144-158) or from an
 * in-memory grid by vpt_nanovdb_grid_info (GridData / TreeData / RootData, NanoVDB.h:2185-2205,
 * 2501-2507, 2687-2725); fields a source does not hold stay zero. */
typedef struct VptNanoVdbInfo {
    char name[256];
    uint32_t grid_type;           /* NanoVDB GridType; 1 = float, the only type a volume accepts */
    uint32_t grid_class;          /* 1 = level set, 2 = fog volume, ... */
    uint64_t grid_bytes;          /* bytes of the in-memory grid */
    uint64_t file_bytes;          /* bytes of the payload in the file (compressed size) */
    uint64_t active_voxels;
    int32_t index_min[3], index_max[3];  /* inclusive index box of the active values */
    double world_min[3], world_max[3];   /* world box: the clip box of the volume */
    double voxel_size[3];
    float map_mat_f[9], map_inv_mat_f[9], map_vec_f[3];  /* index-to-world map, float copy */
    double map_mat_d[9], map_vec_d[3];                    /* index-to-world map, double copy */
    float background;
    uint32_t node_count[3];       /* leaf, lower and upper internal nodes */
    uint32_t tile_count[3];       /* active tiles of those levels */
    /* file only */
    uint32_t codec;               /* 0 = none, 1 = ZIP, 2 = BLOSC */
    uint32_t grid_count;          /* grids in the file */
    uint64_t payload_offset;      /* absolute byte offset of the grid's payload */
    /* in-memory only: the leaf cells a volume built from this grid holds */
    int32_t extent_min[3], extent_max[3];  /* leaf-aligned index box [min, max) */
    int64_t flat_leaves;
} VptNanoVdbInfo;

/* Metadata of grid number `grid_index` (counted over all segments) of an .nvdb file. Host only. */
int vpt_nvdb_file_info(const char* path, uint64_t grid_index, VptNanoVdbInfo* info);
/* Metadata of a NanoVDB grid held in host memory (the buffer of a nanovdb::GridHandle). Host only. */
int vpt_nanovdb_grid_info(const void* grid, uint64_t bytes, VptNanoVdbInfo* info);
/* The leaves a volume built from this float grid holds, decoded on the host: every leaf of the
 * tree inside the extent, then one constant 8^3 leaf per cell of each non-zero tile, then (for
 * a non-zero background) one leaf per cell no root entry covers. leaf_origins gets 3 index
 * coordinates per leaf, leaf_values 512 values per leaf (order x<<6 | y<<3 | z). With both
 * pointers NULL only *count is set; otherwise capacity must be >= the count. Host only. */
int vpt_nanovdb_decode_leaves(const void* grid, uint64_t bytes, int64_t capacity, int32_t* leaf_origins,
                              float* leaf_values, int64_t* count);
/* Density volume from a NanoVDB float grid in host memory: replaces Scene::allocateVolumeGrid
 * (renderer/renderer_scene.cpp:491-537). The clip box is the grid's world box converted to
 * float (:517-519); the global majorant is the maximum over index coordinates [min, max) of
 * the index box (:498-509); lookups follow the grid's map (uniform scale + translation only;
 * other maps are rejected). The tree is flattened into the tracer's 8^3 leaves over the
 * leaf-aligned extent [index_min - 2, index_max + 2]. */
int vpt_set_volume_nanovdb(VptContext* ctx, const void* grid, uint64_t bytes);
/* The same from grid number `grid_index` of an uncompressed .nvdb file: replaces
 * nanovdb::io::readGrid (ext/nanovdb/nanovdb/util/IO.h:576-606) as called at
 * renderer/renderer_scene.cpp:2468. A ZIP or BLOSC grid is refused with an error naming the
 * codec: inflate its payload on the host and call vpt_set_volume_nanovdb. */
int vpt_set_volume_nvdb_file(VptContext* ctx, const char* path, uint64_t grid_index);

/* ---- surfaces ----------------------------------------------------------------------- */
/* Triangle meshes around and inside the volume: the reference's surface path without OptiX
 * (closest and any hits through a BVH built on the host, renderer_kernel_common.h:72-294 and
 * optix_pathtracing_kernels.cu:84-96, 176-195, 216-239, 268-275, 340-356).
 *
 * Scene structure as in renderer/renderer_scene.h: a geometry instance is a triangle mesh
 * with one material; a geometry group is a contiguous range of geometry instances; an
 * instance places a group with a 3x4 transform (several instances may share a group).
 *
 * Materials hold the immediate values of the reference's 1x1 textures: colours in [0, 1] are
 * stored as 8-bit values (truncated, renderer_scene.cpp:860-900) and read back sRGB-decoded;
 * roughness and metallic are 8-bit values read back linearly; emittance is an HDR float RGB
 * (zero = not an emitter). SIMPLE_PBR is what the reference creates for every loaded mesh and
 * rectangle (renderer_scene.cpp:1202-1255, 1411-1414, 1561-1563): SimplePBR_BRDF with
 * reflectance 0.5 and smoothness min(1 - roughness, 0.999) (common_renderer_types.h:1924-1985);
 * LAMBERT is its forceLambertBRDF alternative (:1483-1541). Image textures, normal maps and
 * opacity are not supported. */
#define VPT_MATERIAL_SIMPLE_PBR 0
#define VPT_MATERIAL_LAMBERT 1
typedef struct VptSurfaceMaterial {
    int32_t kind;           /* VPT_MATERIAL_* */
    float base_color[3];    /* SIMPLE_PBR base colour / LAMBERT reflectance (sRGB-encoded) */
    float roughness;        /* SIMPLE_PBR: occlusion_roughness_metallic.y (default 0.5) */
    float metallic;         /* SIMPLE_PBR: occlusion_roughness_metallic.z */
    float emittance[3];     /* linear HDR emittance; all zero = no emitter */
} VptSurfaceMaterial;
/* One geometry instance: object-space vertices (9 floats each: position, shading normal,
 * tangent) and triangles (3 vertex indices each). */
typedef struct VptSurfaceGeometry {
    const float* vertices;
    uint32_t num_vertices;
    const uint32_t* triangles;
    uint32_t num_triangles;
    uint32_t material;
} VptSurfaceGeometry;
/* One instance: the group [first_geometry, first_geometry + num_geometries) placed by the
 * row-major 3x4 object-to-world transform. The light distribution over instances weighs each
 * by the squared length of the transform's first column (compute_light_probs.cu:88-99); the
 * density of reaching an emitter uses uniform_scale, the instance's own scale without the
 * mesh's static transform (Instance::uniformScale, renderer_scene.h:885-898). Normally both
 * are the same number. */
typedef struct VptSurfaceInstance {
    uint32_t first_geometry;
    uint32_t num_geometries;
    float transform[12];
    float uniform_scale;
} VptSurfaceInstance;
/* Replaces the context's surfaces (all three arrays HOST memory; num_instances = 0 removes
 * them). Transforms the vertices to world space, builds the BVH and the light distributions
 * of the emitting triangles (per triangle luminance(emittance) x object-space area, per
 * geometry instance, per instance the group's total x scale^2: compute_light_probs.cu:19-137,
 * renderer_scene.cpp:353-468) and widens the world box (compute_light_probs.cu:139-157).
 * Plain launches of a context with surfaces run the surface tracer (reference and
 * configuration modes, either stream layout; not the wavefront tracer, not leaf staging, not
 * the radiance-cache passes). With surfaces a volume is optional (vpt_clear_volume). */
int vpt_set_surfaces(VptContext* ctx, const VptSurfaceMaterial* materials, uint32_t num_materials,
                     const VptSurfaceGeometry* geometries, uint32_t num_geometries,
                     const VptSurfaceInstance* instances, uint32_t num_instances);
/* Counts of the current surfaces: world triangles, BVH nodes, emitting triangles, and the
 * world box (6 floats: min, max) the launches use. Any pointer may be NULL. */
int vpt_get_surface_info(VptContext* ctx, uint32_t* triangles, uint32_t* bvh_nodes, uint32_t* emitters,
                         float* world_box);
/* Removes the density volume (a surface-only scene: the reference without a density grid). */
int vpt_clear_volume(VptContext* ctx);

/* Image-based environment from an RGB float image (row-major, rows = polar angle from +y).
 * Builds the hierarchical importance map on the device (compute_light_probs.cu:161-211). */
int vpt_set_environment_rgb(VptContext* ctx, const float* host_rgb, int32_t width, int32_t height);
/* Reads the importance mip chain back (size returned by vpt_get_importance_map_info). */
int vpt_get_importance_map_info(VptContext* ctx, int32_t* map_w, int32_t* map_h, int32_t* num_mips,
                                int64_t* total_texels, float* integral);
int vpt_download_importance_map(VptContext* ctx, float* host_mips);

/* Hosek-Wilkie sky texture (renderer/gpu_kernels/analytic_sky_kernels.cu:220-276) from
 * per-band model states computed on the host (16 bands). `states` holds, per band:
 * configs[11][9], radiances[11], emission_correction_factor_sky[11], solar_radius (122 floats);
 * `solar` holds the model's solar-disc data (VPT_SKY_SOLAR_FLOATS floats): the weight of the
 * upper of the two integer turbidities around the requested turbidity, then for each of the 11
 * model channels (320..720 nm) the model's direct-radiance tables of the lower and of the upper
 * turbidity (45 pieces x 4 cubic coefficients each, in the model's order), then the 6
 * limb-darkening coefficients per channel; the direct solar radiance is evaluated at each disc
 * texel's own elevation (analytic_sky_kernels.cu:69-214). `cmf` holds xs[16], ys[16], zs[16],
 * center wavelengths[16] and the CMF integral (65 floats). include_solar_disc = 0 leaves the
 * disc out (the configurations model the sun as a separate delta light; `solar` is then unread). */
#define VPT_SKY_SOLAR_FLOATS (1 + 11 * 2 * 180 + 11 * 6)
int vpt_generate_sky(VptContext* ctx, int32_t width, int32_t height, const float* states,
                     const float* solar, const float* cmf, const float sun_direction[3],
                     int32_t include_solar_disc);
int vpt_download_environment(VptContext* ctx, float* host_rgb);

/* ---- per-frame parameters ----------------------------------------------------------- */
int vpt_set_frame_params(VptContext* ctx, const VptFrameParams* params);

/* ---- plain path tracing (pathTrace raygen, optix_pathtracing_kernels.cu:438-440) -------- */
/* Traces `spp` samples per pixel, continuing each pixel's PCG32 stream, and accumulates
 * into the FP64 sum buffer and the reference's FP32 running mean (numAccumFrames counts
 * previous samples). Persistent kernel, one CTA set per SM, pixels handed out dynamically. */
int vpt_launch_plain(VptContext* ctx, void* stream, uint32_t spp);
/* Same as vpt_launch_plain, additionally writing a per-sample decision record (4 x u32:
 * path vertices, primary lookups, shadow lookups, end code) to a device buffer of
 * width*height*spp*4 u32, sample s of pixel p at (p*spp + s). */
int vpt_launch_plain_logged(VptContext* ctx, void* stream, uint32_t spp, uint32_t* dev_log);

/* Allocation-free launch of the plain tracer. It has no counterpart in the reference: it is for
 * callers that cannot call cudaMalloc (a host renderer whose device memory belongs to its own
 * pool allocator, or code running where allocating is not allowed), so it needs no VptContext.
 * The caller passes every input (grid, majorant grid, environment, importance mip chain, per
 * pixel PCG32 seed states) and output (FP64 sums, FP32 mean) as device pointers, in the layouts
 * the context uses. The launch's scratch memory (work counter, counters, error word and the
 * table of RNG jump constants, 65,792 bytes) is a file-scope __device__ array that every GPU
 * loading the library holds until exit; it is cleared at the start of each call. Limits: spp per
 * call <= VPT_NOALLOC_MAX_SPP (larger requests fail with VPT_ERR_INVALID_ARGUMENT). All calls
 * share the one array, so calls that overlap on the GPU race. The first call with a device
 * current looks the array's address up (cudaGetSymbolAddress): make it before any stream
 * capture. The address is looked up again when the device's current context changes (after
 * cudaDeviceReset, for instance). Device error bits (VPT_DEVERR_*: a segment's step cap, a
 * non-finite sample) are ORed into `device_errors` when the caller gives that word; work
 * counters of these launches are not reported.
 *
 * Buffer layouts (the ones a VptContext builds; x is the slowest axis everywhere):
 *   leaf_table   lx*ly*lz int32 slots (lx = ceil(nx / 8), the same for y and z), the slot of
 *                leaf cell (cx, cy, cz) at (cx*ly + cy)*lz + cz; -1 = empty leaf (density 0)
 *   leaf_values  512 floats per non-empty slot, voxel (x, y, z) of the leaf at x<<6 | y<<3 | z
 *   majorants    mx*my*mz floats, cell (cx, cy, cz) at (cx*my + cy)*mz + cz; a cell covers
 *                2^max(3, majorant_cell_log2) voxels per axis and holds the max density over
 *                its voxels plus one voxel below and two above on each axis
 *   env_texels   env_h rows of env_w float4 (R, G, B, unused), row y = polar angle from +y
 *   imp_mips     num_mips levels back to back, level l = max(map_w>>l, 1) x max(map_h>>l, 1)
 *                floats, row-major; level 0 is the map_w x map_h importance map and the last
 *                level is 1x1 (map_w, map_h: the next powers of two of env_w, env_h). */
#define VPT_NOALLOC_MAX_SPP 4096u
typedef struct VptNoAllocTrace {
    VptFrameParams frame;
    int32_t width, height;
    uint32_t spp;
    uint32_t accum_base;        /* samples already in sum/mean (numAccumFrames of the first) */
    uint32_t stream_base;       /* sample-parallel streams: index of the first sample */
    const int32_t* leaf_table;  /* ceil(n/8)^3 slots, -1 = empty leaf */
    const float* leaf_values;   /* 512 values per slot, order x<<6 | y<<3 | z */
    const float* majorants;     /* mx*my*mz cells of 2^frame.majorant_cell_log2 voxels */
    int32_t nx, ny, nz;
    int32_t mx, my, mz;
    float voxel_size;
    float origin[3];
    float global_majorant;
    const float* env_texels;    /* env_w * env_h float4 (RGB + unused) */
    int32_t env_w, env_h;
    const float* imp_mips;      /* importance mip chain, levels back to back */
    int32_t map_w, map_h, num_mips;
    float imp_integral;
    uint64_t* rng;              /* width*height seed states */
    double* sum_rgb;            /* 3 per pixel */
    float* mean_rgb;            /* 3 per pixel */
    uint32_t* device_errors;    /* optional device word receiving VPT_DEVERR_* bits, or NULL */
} VptNoAllocTrace;
int vpt_launch_plain_noalloc(const VptNoAllocTrace* args, void* stream);
/* ---- image output -------------------------------------------------------------------- */
#define VPT_SDR_SRGB 0x1u     /* sRGB gamma before the 8-bit conversion (the headless default) */
#define VPT_SDR_FLIP_Y 0x2u   /* write rows bottom-up */
/* Tone map of the accumulated mean image, replacing the applyToneMap kernel
 * (renderer/gpu_kernels/post_process_kernels.cu:10-41: per channel x^(1/0.6), then the colour
 * scaled by (1 - exp(-brightness * lum)) / lum; the reference's brightness is 1), fused with the
 * 8-bit conversion of saveImage (common/common_host.cpp:517-568) as the headless loop sets it
 * up (renderer/renderer_main.cpp:1490-1495: no second tone map, negatives clamped to 0, sRGB
 * gamma, min(uint(v * 255), 255) per channel, alpha 255). dev_rgba32 receives width*height
 * float4 (the reference's outputBuffer, alpha 1), dev_rgba8 width*height 32-bit RGBA words
 * (R in the low byte); either may be NULL. Asynchronous on `stream`. */
int vpt_tonemap(VptContext* ctx, void* stream, float brightness, uint32_t sdr_flags, float* dev_rgba32,
                uint32_t* dev_rgba8);
/* The same into a context-owned device image, copied to host_rgba8 (width*height words):
 * the frame enqueueSaveImage writes to "%03u.png" (renderer_main.cpp:1646-1655). Synchronous. */
int vpt_download_image_rgba8(VptContext* ctx, float brightness, uint32_t sdr_flags, uint32_t* host_rgba8);
int vpt_reset_accumulation(VptContext* ctx);

/* Reads back the accumulation: FP64 per-pixel RGB sums and sample count, FP32 running mean. */
int vpt_download_sum(VptContext* ctx, double* host_rgb, uint32_t* num_samples);
int vpt_download_mean(VptContext* ctx, float* host_rgb);
/* Device pointers of the accumulation buffers (FP64 sum, FP32 mean; 3 values per pixel). */
int vpt_get_accum_device_ptrs(VptContext* ctx, double** dev_sum, float** dev_mean);

/* Work counters of the launches since the last reset: density lookups, path vertices,
 * samples, majorant-grid cell steps. Read back with a synchronisation. */
int vpt_get_counters(VptContext* ctx, uint64_t* lookups, uint64_t* vertices, uint64_t* samples,
                     uint64_t* cell_steps);
int vpt_reset_counters(VptContext* ctx);
uint32_t vpt_get_device_errors(VptContext* ctx);
int vpt_synchronize(VptContext* ctx, void* stream);

/* Tracker of vpt_launch_plain: kind 0 = persistent megakernel (the default: one launch,
 * asynchronous, capturable in a CUDA graph), 1 = wavefront: an event kernel and a persistent
 * tracking kernel alternate in passes over per-slot path state, the host issuing passes until
 * every slot retired, so the call returns once the launch's work is nearly done; a stream under
 * graph capture always gets the megakernel. slots_per_sm (paths in flight per SM, 0 = 3072),
 * pass_steps (lookups a segment may take per pass, 0 = 64) and track_ctas_per_sm (0 = as many
 * as fit) tune the wavefront. Both trackers draw each path's random numbers in the same order. */
int vpt_set_tracker(VptContext* ctx, int32_t kind, int32_t slots_per_sm, int32_t pass_steps,
                    int32_t track_ctas_per_sm);
/* Leaf staging of the persistent tracker (majorant-grid mode on sample-parallel streams, and its
 * logged form): each warp keeps one 8^3 leaf in shared memory, brought in with one bulk
 * asynchronous copy (cp.async.bulk) whenever at least `min_lanes` of its lanes look up inside
 * the same leaf in one tracking step; those lanes read their stencils from it. 0 = off (the
 * default). Decisions and values are those of the unstaged tracker. */
int vpt_set_leaf_staging(VptContext* ctx, int32_t min_lanes);
/* Launch shape of the persistent tracker (CTAs per SM, threads per CTA, a multiple of 32 up to
 * 128) and the number of parked lanes of a warp that triggers its joint event phase; 0 = defaults:
 * one CTA of 896 threads per SM for the plain tracer on sample-parallel streams and for the
 * radiance-cache passes without meshes, as many 128-thread CTAs as fit for the other forms; park
 * threshold 16 for the plain tracer, 24 for the radiance-cache passes. Contexts whose launches run
 * concurrently on one GPU (several scenes at once) do better with 128-thread CTAs, which can share
 * an SM. */
int vpt_set_launch_shape(VptContext* ctx, int32_t ctas_per_sm, int32_t threads_per_cta,
                         int32_t park_threshold);

/* ---- Neural radiance cache passes (renderer/renderer_main.cpp:1553-1637) ----------------
 * The training and render passes of the tracer, the set-up kernels between them, and one call
 * that runs a whole frame with a cache from rtc8_nrc.h. Buffers follow the reference's
 * (renderer/renderer_main.cpp:197-230): RadianceQuery records of 14 floats (inference buffer
 * roundUp(w*h, 128) records, training buffers 2 x 2^17), TerminalInfo / TrainingVertexInfo
 * records of 16 bytes, training-suffix terminals of 4 bytes, predictions of 3 floats. The
 * training image size and the number of training vertices stay on the device. The world box of
 * the queries is the density grid's box (a volume-only scene, compute_light_probs.cu:139-157). */
#define VPT_NRC_TRAIN_DATA_PER_FRAME 65536u  /* numTrainingDataPerFrame (renderer_shared.h:12) */
#define VPT_NRC_TRAIN_BUFFER_SIZE 131072u    /* trainBufferSize (renderer_shared.h:13) */
#define VPT_NRC_QUERY_FLOATS 14

typedef struct VptNrcBuffers {
    float* infer_query;          /* inferenceRadianceQueryBuffer: infer_capacity x 14 */
    void* infer_terminal;        /* inferenceTerminalInfoBuffer: w*h x {float tp[3]; u32 bits} */
    uint32_t* train_suffix;      /* trainSuffixTerminalInfoBuffer: w*h */
    float* inferred;             /* inferredRadianceBuffer: infer_capacity x 3 */
    float* frame_contribution;   /* perFrameContributionBuffer: w*h x 3 */
    float* train_query[2];       /* trainRadianceQueryBuffer[0..1]: 2^17 x 14 */
    float* train_target[2];      /* trainTargetBuffer[0..1]: 2^17 x 3 */
    void* train_vertex;          /* trainVertexInfoBuffer: 2^17 x {float tp[3]; u32 bits} */
    float* train_end_query;      /* end queries of the training suffixes: w*h x 14 (the reference
                                    shares the render pass's inference buffer) */
    float* train_end_inferred;   /* their predictions: w*h x 3 */
    uint64_t* train_rng;         /* training-pass PCG32 states when rng_stream_mode = 1 */
    uint32_t* shufflers;         /* dataShufflerBuffer: 2^16 LCG states */
    uint32_t* counters;          /* [0..1] numTrainingData, [2..5] trainImageSize (x, y) per
                                    buffer, [6] offsetToSelectUnbiasedPath, [7] training-pass
                                    queries (trainW * trainH), [8..15] unused */
    float* stats;                /* per buffer: targetMinMax (min rgb, max rgb), targetAvg */
    uint32_t infer_capacity;
    uint32_t buffer_index;       /* nrcBufferIndex of the last training iteration */
    uint32_t render_spp;         /* sample slots per pixel of the render-pass buffers (records of
                                    sample s of pixel p at s * w * h + p) */
} VptNrcBuffers;

/* Allocates the cache buffers (once per context; the shufflers start from the LCG seeded with
 * 471313181, renderer_main.cpp:218-229). Called implicitly by the entry points below. */
int vpt_nrc_enable(VptContext* ctx);
int vpt_nrc_get_buffers(VptContext* ctx, VptNrcBuffers* out);
/* Whether the query's roughness slot carries the local density / density_coeff (for the volume
 * encoding of rtc8_nrc.h; the reference writes roughness 0 in a medium, 0 = that). The cache's
 * target scale is VptFrameParams.radiance_scale. */
int vpt_nrc_set_query_density(VptContext* ctx, int32_t query_density);
/* Path-spread termination factors (pathTerminationFactor c, renderer_shared.h:11): a render path
 * ends with a cache query once its spread exceeds render_factor times the primary footprint, a
 * biased training suffix at train_factor (optix_pathtracing_kernels.cu:282-289 uses c and 2c).
 * render_factor 0 = the reference's 0.01; train_factor 0 = 2 x render_factor. */
int vpt_nrc_set_termination_factor(VptContext* ctx, float render_factor, float train_factor);
/* prepareNRC(offsetToSelectUnbiasedPath, isNewSequence) on training buffer `buffer_index`
 * (nrc_set_up_kernels.cu:4-44). */
int vpt_prepare_nrc(VptContext* ctx, void* stream, uint32_t buffer_index, uint32_t offset, int32_t new_sequence);
/* generateTrainingData on the training image of buffer `buffer_index`. */
int vpt_launch_generate_training(VptContext* ctx, void* stream, uint32_t buffer_index);
/* propagateRadianceValues (nrc_set_up_kernels.cu:46-86), reading the cache's predictions for
 * the training-pass queries from `inferred`. */
int vpt_propagate(VptContext* ctx, void* stream);
/* shuffleTrainingData (nrc_set_up_kernels.cu:88-174) of buffer `buffer_index` into buffer 1. */
int vpt_shuffle(VptContext* ctx, void* stream, uint32_t buffer_index);
/* pathTraceWithNRC on the full image: one sample per pixel. */
int vpt_launch_render_nrc(VptContext* ctx, void* stream);
/* accumulateInferredRadianceValues (nrc_set_up_kernels.cu:176-219) as sample number
 * `accum_frames` of the FP32 running mean, also added to the FP64 sums; the context's sample
 * count becomes accum_frames + 1. */
int vpt_accumulate_inferred(VptContext* ctx, void* stream, uint32_t accum_frames);
/* GB300 form of the render passes of one frame: `spp` samples per pixel in ONE persistent launch
 * on sample-parallel streams (VptFrameParams.rng_stream_mode must be 1; the reference runs one
 * launch per sample on per-pixel streams, renderer_main.cpp:1617-1637). The render-pass buffers
 * grow to `spp` slots per pixel (the first call with a larger spp synchronises the device). */
int vpt_launch_render_nrc_batch(VptContext* ctx, void* stream, uint32_t spp);
/* Accumulation of the `spp` samples of a batched render pass: FP64 sums, and the mean as the sum
 * over accum_frames + spp samples (which becomes the context's sample count). */
int vpt_accumulate_inferred_batch(VptContext* ctx, void* stream, uint32_t accum_frames, uint32_t spp);
/* One frame of renderer_main.cpp:1553-1637 with the cache `nrc` (an NrcHandle* of
 * rtc8_nrc.h): `train_iterations` x (prepareNRC with the next offset of mt19937(72139121) and
 * isNewSequence = new_sequence, training pass, inference on its queries, propagation, shuffle,
 * 4 training steps of 16384 records), then `spp` x (render pass, inference, accumulation), or,
 * with sample-parallel streams (rng_stream_mode 1), one batched render pass of `spp` samples,
 * one inference and one accumulation.
 * Accumulation continues the context's (the reference restarts it every frame: call
 * vpt_reset_accumulation first for that). Nothing is synchronised. With sample-parallel streams
 * the first training pass and the frame's render samples are ONE persistent launch (training
 * pixels first, then render samples: lanes that finish a training suffix go on with render
 * samples, so the longest suffixes hold no idle SM slots); the training pass then draws from its
 * own per-pixel states (train_rng) so the two kinds of work share no state. The render queries
 * are inferred after the training steps, with the updated network, as in the reference. */
int vpt_nrc_frame(VptContext* ctx, void* nrc, void* stream, uint32_t train_iterations, uint32_t spp,
                  int32_t new_sequence);
/* 1 (default): the combined training + render launch of vpt_nrc_frame described above; 0: the
 * first training pass and the batched render pass as two launches (smaller kernels each). */
int vpt_nrc_set_combined_pass(VptContext* ctx, int32_t on);

#ifdef __cplusplus
}
#endif

#endif /* RTC8_VPT_H */
