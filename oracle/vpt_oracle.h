/*
 * ORACLE (test infrastructure only) — CPU restatement of the reference path tracer's
 * volume-only hot path (shocker-0x15/rtcamp8). Only tests/, the smoke check and the
 * CPU-baseline / reference legs of bench.py load this library; the product library never
 * links, calls or ships it.
 *
 * Parity status: the reference's own hot path (an OptiX ray-generation program plus
 * tiny-cuda-nn) cannot be built in this environment, and the reference has no tests or
 * golden vectors. The oracle is therefore pinned component by component against programs
 * compiled from the reference's own sources (NanoVDB sampler / ray clip, basic_types.h
 * math, Hosek-Wilkie sky model) through the committed recipe in oracle/build_ref.sh and
 * the golden vectors in tests/golden/; the end-to-end estimator is pinned by analytic
 * tests (furnace, constant-density transmittance) only.
 *
 * All structs are plain C so Python (ctypes) can fill them.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OrcScene {
    /* Dense voxel array, x-major (index = (x * ny + y) * nz + z), values outside are 0. */
    const float* voxels;
    int32_t nx, ny, nz;
    float inv_voxel_size;      /* world -> index scale (float copy of 1/voxel size) */
    float origin[3];           /* world position of index (0,0,0) */
    float bbox_min[3], bbox_max[3];   /* world-space clip box of the grid */
    float global_majorant;     /* max voxel value (reference loop over [min,max)) */
    const float* cell_majorant;       /* per 8^3-voxel cell, 9^3 apron max; may be null */
    int32_t cx, cy, cz;
    float density_coeff;
    float albedo;
    int32_t phase_kind;        /* 0 = Schlick(k), 1 = Henyey-Greenstein(g) */
    float phase_param;

    /* Image-based environment (point-sampled RGB, row-major, y = polar angle). */
    int32_t env_enabled;
    const float* env_rgb;      /* env_w * env_h * 3 */
    int32_t env_w, env_h;
    float env_power, env_rotation;
    const float* imp_mips;     /* importance mip chain, level L at imp_offsets[L] */
    const int64_t* imp_offsets;
    int32_t map_w, map_h, num_mips;
    float imp_integral;

    /* Directional sun (config mode only). */
    int32_t sun_enabled;
    float sun_dir[3];          /* unit vector towards the sun */
    float sun_irradiance[3];
    float sun_prob;            /* probability of picking the sun in NEE */

    float world_radius;
    float world_min[3], world_max[3];

    float cam_aspect, cam_fovy;
    float cam_pos[3];
    float cam_quat[4];         /* x, y, z, w */
    int32_t width, height;

    int32_t max_bounces;       /* 0 = unlimited */
    int32_t rr_start;          /* RR draws when pathLength >= rr_start */
    int32_t majorant_mode;     /* 0 = single global majorant, 1 = per-cell majorant DDA */
    int32_t max_steps;         /* safety cap on density lookups per segment, 0 = none */
    int32_t stream_mode;       /* 0 = per-pixel sequential streams, 1 = sample s jumped by s * 2^40 */
    int32_t maj_shift;         /* majorant cells of 2^maj_shift voxels (cell_majorant has cx*cy*cz) */
    float shadow_rr;           /* Russian-roulette threshold of shadow-ray visibility, 0 = off */
    /* Triangle meshes (orc_surfaces_create), NULL = volume-only scene; plain passes only. */
    const struct OrcSurfaces* surfaces;
    int32_t volume_disabled;   /* 1: no density grid (surfaces only) */
} OrcScene;

/* Surface scene inputs, laid out like the product's VptSurface* structs: materials with the
 * immediate texture values, geometry instances with object-space vertices (position, normal,
 * tangent) and triangles, instances with a row-major 3x4 transform over a geometry range. */
typedef struct OrcSurfMaterial {
    int32_t kind;              /* 0 = SimplePBR, 1 = Lambert */
    float base_color[3];
    float roughness, metallic;
    float emittance[3];
} OrcSurfMaterial;
typedef struct OrcSurfGeometry {
    const float* vertices;
    uint32_t num_vertices;
    const uint32_t* triangles;
    uint32_t num_triangles;
    uint32_t material;
} OrcSurfGeometry;
typedef struct OrcSurfInstance {
    uint32_t first_geometry, num_geometries;
    float transform[12];
    float uniform_scale;
} OrcSurfInstance;
typedef struct OrcSurfaces OrcSurfaces;

/* Per-sample decision record: vertices, primary lookups, shadow lookups, end code. */
enum {
    ORC_END_ESCAPE = 1,
    ORC_END_RR = 2,
    ORC_END_PDF_ZERO = 3,
    ORC_END_MAX_BOUNCES = 4,
    ORC_END_STEP_CAP = 5,
    ORC_END_CACHE = 6,       /* radiance-cache passes: ended with a cache query */
    ORC_END_TRAIN_FULL = 7,  /* training pass: the training-vertex buffer was full */
};

/* Radiance-cache pass constants (renderer_shared.h:11-13, 74) and outputs. */
#define ORC_NRC_INVALID_VERTEX 0x003FFFFFu
#define ORC_NRC_TRAIN_BUFFER_SIZE 131072u
#define ORC_NRC_TERMINATION_FACTOR 0.01f
#define ORC_NRC_QUERY_FLOATS 14
typedef struct OrcNrcSink {
    int32_t mode;              /* 1 = pathTraceWithNRC, 2 = generateTrainingData */
    int32_t density_query;     /* roughness slot = local density / density_coeff */
    uint32_t img_w, img_h;     /* pass image (training image size in mode 2) */
    uint32_t unbiased_offset;  /* offsetToSelectUnbiasedPath */
    float termination;         /* path-spread termination factor (0 = 0.01) */
    float train_termination;   /* biased training suffixes (0 = 2 x termination) */
    float* infer_query;        /* 14 per pass pixel */
    float* terminal_tp;        /* mode 1: 3 per pixel */
    uint32_t* terminal_bits;   /* mode 1: hasQuery | pathLength << 1 */
    float* frame_contribution; /* mode 1: 3 per pixel */
    uint32_t* train_suffix;    /* mode 2: per pixel, prev | hasQuery << 22 | pathLength << 23 | unbiased << 31 */
    float* train_query;        /* mode 2: 14 per vertex */
    float* train_target;       /* mode 2: 3 per vertex */
    float* train_local_tp;     /* mode 2: 3 per vertex */
    uint32_t* train_bits;      /* mode 2: prev | pathLength << 22 | unbiased << 30 */
    uint32_t* num_train;       /* mode 2: vertex counter (numTrainingData) */
} OrcNrcSink;

int orc_version(void);

/* PCG32 / seeding helpers. */
void orc_seed_states(int32_t width, int32_t height, uint64_t seed, uint64_t* out);
void orc_pcg_floats(uint64_t state, int32_t n, float* out, uint64_t* state_out);

/* Importance map build for an RGB environment image (restates computeFirstMip... +
 * computeMipOfImportanceMap). Writes the chain into mips_out (size from orc_imp_map_size). */
int64_t orc_imp_map_size(int32_t env_w, int32_t env_h, int32_t* map_w, int32_t* map_h,
                         int32_t* num_mips, int64_t* offsets);
float orc_build_imp_map(const float* env_rgb, int32_t env_w, int32_t env_h, float* mips_out);

/* Majorant cells (per 8^3 cell, max over voxels [8c-1, 8c+9]) and the return value is the
 * reference's global majorant (max over index coordinates [0, n-1) per axis). */
float orc_majorants(const float* voxels, int32_t nx, int32_t ny, int32_t nz, float* cells);

/* Component batch entry points used by the known-answer tests. */
void orc_sample_density(const OrcScene* sc, const float* idx_xyz, int32_t n, float* out);
void orc_srgb_gamma(const float* in, int32_t n, float* out);
/* Tone map + 8-bit sRGB conversion of a mean image (n RGB pixels) into out_rgb (3 floats per
 * pixel) and out_rgba (4 bytes per pixel); either may be NULL. */
void orc_tonemap(const float* mean, int32_t n, float brightness, int32_t srgb, float* out_rgb, uint8_t* out_rgba);
void orc_clip_rays(const OrcScene* sc, const float* org, const float* dir, int32_t n,
                   float* t0, float* t1, int32_t* hit);
void orc_env_sample(const OrcScene* sc, const float* u, int32_t n, float* dir, float* pdf,
                    float* rgb);
void orc_env_evaluate(const OrcScene* sc, const float* dir, int32_t n, float* pdf, float* rgb);
void orc_imp_sample(const OrcScene* sc, const float* u, int32_t n, float* out5);
/* Prepared surfaces (world triangles, light distributions) from the raw inputs; box_out gets
 * the union of the instances' transformed boxes (min, max). NULL for invalid input. */
OrcSurfaces* orc_surfaces_create(const OrcSurfMaterial* materials, uint32_t num_materials,
                                 const OrcSurfGeometry* geometries, uint32_t num_geometries,
                                 const OrcSurfInstance* instances, uint32_t num_instances, float* box_out);
void orc_surfaces_destroy(OrcSurfaces* s);
/* Closest hits (tri index or -1, t, b1, b2 per ray) and any-hit tests of n rays. */
void orc_surface_closest(const OrcSurfaces* s, const float* org, const float* dir, int32_t n, float tmax,
                         int32_t* tri, float* tb);
void orc_surface_any(const OrcSurfaces* s, const float* org, const float* dir, const float* tmax, int32_t n,
                     int32_t* hit);
/* BSDF of a material (kind, decoded parameters) evaluated for n (query, sampled) direction
 * pairs in the shading frame: value (3), pdf (1); and sampled: direction (3), value (3), pdf. */
void orc_bsdf_eval(const OrcSurfMaterial* m, const float* q, const float* v, int32_t n, float* val, float* pdf);
void orc_bsdf_sample(const OrcSurfMaterial* m, const float* q, const float* u, int32_t n, float* out7);
/* offsetRayOrigin of n (point, normal) pairs (6 floats each). */
void orc_offset_origin(const float* pn, int32_t n, float* out);
void orc_phase_sample(int32_t kind, float param, const float* u, int32_t n, float* dir_local,
                      float* pdf);
void orc_phase_eval(int32_t kind, float param, const float* dir_local, int32_t n, float* pdf);
void orc_polar_yup(const float* v, int32_t n, float* theta_phi);
void orc_coordinate_system(const float* nrm, int32_t n, float* tb);
void orc_quat_to_matrix(const float* q, float* m9);

/* Plain path tracer: spp samples per pixel over rows [row0, row1), continuing each
 * pixel's PCG32 stream. sum_rgb (double, += per sample), mean_rgb (reference running
 * mean with numAccumFrames = accum_base + i) and dlog (4 x u32 per pixel-sample,
 * index (pixel * spp + i)) may be null. Returns the number of density lookups. */
int64_t orc_render_plain(const OrcScene* sc, uint64_t* rng, int32_t accum_base, int32_t spp,
                         double* sum_rgb, float* mean_rgb, uint32_t* dlog, int32_t row0,
                         int32_t row1, int32_t nthreads);

/* One radiance-cache pass (optix_pathtracing_kernels.cu:31-434, withNRC = true), one sample per
 * pixel of the pass image, continuing the per-pixel PCG32 streams of the full image. dlog (4 x u32
 * per pass pixel) may be null. Returns the number of density lookups. */
int64_t orc_nrc_pass(const OrcScene* sc, uint64_t* rng, const OrcNrcSink* nrc, uint32_t* dlog);

/* Set-up kernels between the passes (nrc_setup_oracle.cpp), on host copies of the buffers:
 * counters (16 u32: numTrainingData[2], trainImageSize[2][2], offset, training queries),
 * stats (per buffer min rgb, max rgb, avg rgb), vertex / terminal records of 4 words. */
void orc_nrc_shufflers(uint32_t* out);
void orc_nrc_prepare(uint32_t* counters, float* stats, uint32_t* train_suffix, int32_t width, int32_t height,
                     uint32_t buf, uint32_t offset, int32_t new_sequence);
void orc_nrc_propagate(uint32_t num_suffixes, const uint32_t* train_suffix, const float* inferred,
                       const float* infer_query, const float* vertex, const float* train_query0,
                       float* train_target0, float radiance_scale);
void orc_nrc_shuffle(uint32_t num_training, float* stats_buf, uint32_t* shufflers, const float* train_query0,
                     const float* train_target0, float* train_query1, float* train_target1,
                     float radiance_scale, uint32_t* writers);
void orc_nrc_accumulate(uint32_t num_pixels, const float* terminal, const float* frame_contribution,
                        const float* inferred, const float* infer_query, float radiance_scale,
                        uint32_t accum_frames, double* sum, float* mean);

#ifdef __cplusplus
}
#endif
