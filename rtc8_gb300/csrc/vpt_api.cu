// C ABI of the volumetric path tracer: context, scene upload, frame parameters, launches.
// The context plays the role of the reference's launch-parameter blocks
// (renderer/renderer_shared.h:113-172) and the buffers set up in
// renderer/renderer_main.cpp:80-129 and :197-297.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/rtc8_vpt.h"
#include "vpt_ctx.h"
#include "vpt_scene.cuh"
#include "vpt_tracer.cuh"

namespace {

thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define VPT_CUDA(call)                                                                         \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return set_error(VPT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
int dev_alloc(T** p, size_t count) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (count == 0) return VPT_OK;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
    if (e != cudaSuccess) return set_error(VPT_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return VPT_OK;
}

template <typename T>
void dev_free(T** p) {
    if (*p) cudaFree(*p);
    *p = nullptr;
}

}  // namespace

namespace vpt {
int ctx_set_error(int code, const char* msg) { return set_error(code, msg); }
}  // namespace vpt

using vpt::VptContextImpl;

extern "C" {

const char* vpt_last_error(void) { return g_last_error.c_str(); }

int vpt_create(int32_t w, int32_t h, VptContext** out) {
    if (!out || w <= 0 || h <= 0) return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_create: bad arguments");
    int device = 0, num_sms = 0;
    VPT_CUDA(cudaGetDevice(&device));
    VPT_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
    auto* c = new VptContext();
    c->width = w;
    c->height = h;
    c->device = device;
    c->num_sms = num_sms;
    int64_t npix = static_cast<int64_t>(w) * h;
    int rc;
    if ((rc = dev_alloc(&c->d_rng, npix)) || (rc = dev_alloc(&c->d_sum, 3 * npix)) ||
        (rc = dev_alloc(&c->d_mean, 3 * npix)) || (rc = dev_alloc(&c->d_work, 4)) ||
        (rc = dev_alloc(&c->d_counters, 8)) || (rc = dev_alloc(&c->d_frame, 2)) || (rc = dev_alloc(&c->d_err, 1)) || (rc = dev_alloc(&c->d_scratch_u32, 4)) ||
        (rc = dev_alloc(&c->d_integral, 1))) {
        vpt_destroy(c);
        return rc;
    }
    VPT_CUDA(cudaMemset(c->d_sum, 0, 3 * npix * sizeof(double)));
    VPT_CUDA(cudaMemset(c->d_mean, 0, 3 * npix * sizeof(float)));
    VPT_CUDA(cudaMemset(c->d_counters, 0, 8 * sizeof(unsigned long long)));
    VPT_CUDA(cudaMemset(c->d_frame, 0, 2 * sizeof(uint32_t)));
    VPT_CUDA(cudaMemset(c->d_err, 0, sizeof(unsigned int)));
    // A constant 1x1 environment so that a context is always renderable.
    float one[3] = {1.0f, 1.0f, 1.0f};
    if ((rc = vpt_set_environment_rgb(c, one, 1, 1)) != VPT_OK) {
        vpt_destroy(c);
        return rc;
    }
    if ((rc = vpt_seed_rng(c, 591842031321323413ULL)) != VPT_OK) {
        vpt_destroy(c);
        return rc;
    }
    *out = c;
    return VPT_OK;
}

int vpt_destroy(VptContext* c) {
    if (!c) return VPT_OK;
    c->release_nrc();
    c->release_wf();
    c->release_surfaces();
    dev_free(&c->d_rng);
    dev_free(&c->d_sum);
    dev_free(&c->d_mean);
    dev_free(&c->d_work);
    dev_free(&c->d_counters);
    dev_free(&c->d_frame);
    dev_free(&c->d_err);
    dev_free(&c->d_scratch_u32);
    dev_free(&c->d_integral);
    dev_free(&c->d_leaf_table);
    dev_free(&c->d_leaf_values);
    dev_free(&c->d_cell_maj);
    dev_free(&c->d_maj);
    dev_free(&c->d_jumps);
    dev_free(&c->d_dense);
    dev_free(&c->d_rgba8);
    dev_free(&c->d_env);
    dev_free(&c->d_mips);
    delete c;
    return VPT_OK;
}

int vpt_seed_rng(VptContext* c, uint64_t seed) {
    if (!c) return set_error(VPT_ERR_INVALID_ARGUMENT, "null context");
    int64_t npix = static_cast<int64_t>(c->width) * c->height;
    std::vector<uint64_t> states(npix);
    std::mt19937_64 gen(seed);
    for (int64_t i = 0; i < npix; ++i) states[i] = gen();
    VPT_CUDA(cudaMemcpy(c->d_rng, states.data(), npix * sizeof(uint64_t), cudaMemcpyHostToDevice));
    c->stream_samples = 0;
    VPT_CUDA(cudaMemset(c->d_frame, 0, sizeof(uint32_t)));
    if (int rc = vpt::nrc_reseed_train_rng(c)) return rc;
    return vpt_reset_accumulation(c);
}

int vpt_set_rng_states(VptContext* c, const uint64_t* host) {
    if (!c || !host) return set_error(VPT_ERR_INVALID_ARGUMENT, "null argument");
    int64_t npix = static_cast<int64_t>(c->width) * c->height;
    VPT_CUDA(cudaMemcpy(c->d_rng, host, npix * sizeof(uint64_t), cudaMemcpyHostToDevice));
    return vpt::nrc_reseed_train_rng(c);
}

int vpt_get_rng_states(VptContext* c, uint64_t* host) {
    if (!c || !host) return set_error(VPT_ERR_INVALID_ARGUMENT, "null argument");
    int64_t npix = static_cast<int64_t>(c->width) * c->height;
    VPT_CUDA(cudaDeviceSynchronize());
    VPT_CUDA(cudaMemcpy(host, c->d_rng, npix * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    return VPT_OK;
}

int vpt_reset_accumulation(VptContext* c) {
    if (!c) return set_error(VPT_ERR_INVALID_ARGUMENT, "null context");
    int64_t npix = static_cast<int64_t>(c->width) * c->height;
    VPT_CUDA(cudaMemset(c->d_sum, 0, 3 * npix * sizeof(double)));
    VPT_CUDA(cudaMemset(c->d_mean, 0, 3 * npix * sizeof(float)));
    c->accum_samples = 0;
    VPT_CUDA(cudaMemset(c->d_frame + 1, 0, sizeof(uint32_t)));
    return VPT_OK;
}

// ------------------------------------------------------------------------------ volume
static int build_grid_from_dense(VptContext* c, const float* d_dense, int nx, int ny, int nz, float voxel_size,
                                 const float origin[3]) {
    c->nx = nx;
    c->ny = ny;
    c->nz = nz;
    c->lx = (nx + 7) / 8;
    c->ly = (ny + 7) / 8;
    c->lz = (nz + 7) / 8;
    int64_t cells = static_cast<int64_t>(c->lx) * c->ly * c->lz;
    int32_t* d_active = nullptr;
    int rc;
    if ((rc = dev_alloc(&d_active, cells)) || (rc = dev_alloc(&c->d_cell_maj, cells)) ||
        (rc = dev_alloc(&c->d_leaf_table, cells)))
        return rc;
    vpt::leaf_stats(d_dense, nx, ny, nz, c->lx, c->ly, c->lz, d_active, c->d_cell_maj, 0);
    vpt::global_max(d_dense, nx, ny, nz, c->d_scratch_u32, 0);
    std::vector<int32_t> table(cells);
    VPT_CUDA(cudaMemcpy(table.data(), d_active, cells * sizeof(int32_t), cudaMemcpyDeviceToHost));
    dev_free(&d_active);
    int64_t slots = 0;
    for (int64_t i = 0; i < cells; ++i) table[i] = table[i] ? static_cast<int32_t>(slots++) : -1;
    c->active_leaves = slots;
    c->total_leaves = cells;
    VPT_CUDA(cudaMemcpy(c->d_leaf_table, table.data(), cells * sizeof(int32_t), cudaMemcpyHostToDevice));
    if ((rc = dev_alloc(&c->d_leaf_values, std::max<int64_t>(slots, 1) * 512))) return rc;
    vpt::pack_leaves(d_dense, nx, ny, nz, c->lx, c->ly, c->lz, c->d_leaf_table, c->d_leaf_values, 0);
    unsigned int gmax_bits = 0;
    VPT_CUDA(cudaMemcpy(&gmax_bits, c->d_scratch_u32, sizeof(unsigned int), cudaMemcpyDeviceToHost));
    std::memcpy(&c->global_majorant, &gmax_bits, sizeof(float));
    c->voxel_size = voxel_size;
    c->inv_voxel_size = static_cast<float>(1.0 / static_cast<double>(voxel_size));
    for (int a = 0; a < 3; ++a) c->origin[a] = origin[a];
    int n[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
        c->bbox_min[a] = origin[a];
        c->bbox_max[a] = static_cast<float>(origin[a] + static_cast<double>(n[a]) * voxel_size);
    }
    c->has_volume = true;
    c->update_world_box();
    c->maj_shift = 0;  // the pooled majorant grid is rebuilt at the next launch
    VPT_CUDA(cudaDeviceSynchronize());
    return VPT_OK;
}

int vpt_set_volume_dense(VptContext* c, const float* host, int32_t nx, int32_t ny, int32_t nz, float voxel_size,
                         const float origin[3]) {
    if (!c || !host || nx <= 1 || ny <= 1 || nz <= 1 || !(voxel_size > 0) || !origin)
        return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_set_volume_dense: bad arguments");
    int64_t total = static_cast<int64_t>(nx) * ny * nz;
    int rc;
    if ((rc = dev_alloc(&c->d_dense, total))) return rc;
    VPT_CUDA(cudaMemcpy(c->d_dense, host, total * sizeof(float), cudaMemcpyHostToDevice));
    return build_grid_from_dense(c, c->d_dense, nx, ny, nz, voxel_size, origin);
}

int vpt_set_volume_dense_device(VptContext* c, const float* dev, int32_t nx, int32_t ny, int32_t nz,
                                float voxel_size, const float origin[3]) {
    if (!c || !dev || nx <= 1 || ny <= 1 || nz <= 1 || !(voxel_size > 0) || !origin)
        return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_set_volume_dense_device: bad arguments");
    int64_t total = static_cast<int64_t>(nx) * ny * nz;
    int rc;
    if ((rc = dev_alloc(&c->d_dense, total))) return rc;
    VPT_CUDA(cudaMemcpy(c->d_dense, dev, total * sizeof(float), cudaMemcpyDeviceToDevice));
    return build_grid_from_dense(c, c->d_dense, nx, ny, nz, voxel_size, origin);
}

int vpt_generate_fbm_volume(VptContext* c, int32_t n, uint32_t seed, int32_t octaves, float lacunarity, float gain,
                            float base_frequency, float threshold, float voxel_size, const float origin[3]) {
    if (!c || n <= 1 || n > 4096 || octaves <= 0 || octaves > 16 || !(voxel_size > 0) || !origin || threshold < 0 ||
        threshold >= 1)
        return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_generate_fbm_volume: bad arguments");
    int64_t total = static_cast<int64_t>(n) * n * n;
    int rc;
    if ((rc = dev_alloc(&c->d_dense, total))) return rc;
    vpt::generate_fbm(c->d_dense, n, seed, octaves, lacunarity, gain, base_frequency, threshold, c->d_scratch_u32, 0);
    VPT_CUDA(cudaGetLastError());
    return build_grid_from_dense(c, c->d_dense, n, n, n, voxel_size, origin);
}

int vpt_generate_fbm_union(VptContext* c, int32_t n, uint32_t seed_a, uint32_t seed_b, int32_t octaves,
                           float lacunarity, float gain, float base_frequency, float threshold, float voxel_size,
                           const float origin[3]) {
    if (!c || n <= 1 || n > 4096 || octaves <= 0 || octaves > 16 || !(voxel_size > 0) || !origin || threshold < 0 ||
        threshold >= 1)
        return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_generate_fbm_union: bad arguments");
    int64_t total = static_cast<int64_t>(n) * n * n;
    int rc;
    if ((rc = dev_alloc(&c->d_dense, total))) return rc;
    float* second = nullptr;
    if ((rc = dev_alloc(&second, total))) return rc;
    vpt::generate_fbm(c->d_dense, n, seed_a, octaves, lacunarity, gain, base_frequency, threshold, c->d_scratch_u32, 0);
    vpt::generate_fbm(second, n, seed_b, octaves, lacunarity, gain, base_frequency, threshold, c->d_scratch_u32, 0);
    vpt::max_into(c->d_dense, second, total, 0);
    cudaError_t e = cudaGetLastError();
    dev_free(&second);
    if (e != cudaSuccess) return set_error(VPT_ERR_CUDA, std::string("vpt_generate_fbm_union: ") + cudaGetErrorString(e));
    return build_grid_from_dense(c, c->d_dense, n, n, n, voxel_size, origin);
}

int vpt_download_volume_dense(VptContext* c, float* host) {
    if (!c || !host || !c->d_dense) return set_error(VPT_ERR_NOT_READY, "no dense volume resident");
    int64_t total = static_cast<int64_t>(c->nx) * c->ny * c->nz;
    VPT_CUDA(cudaDeviceSynchronize());
    VPT_CUDA(cudaMemcpy(host, c->d_dense, total * sizeof(float), cudaMemcpyDeviceToHost));
    return VPT_OK;
}

int vpt_get_volume_info(VptContext* c, int64_t* active, int64_t* total, float* gmaj, int64_t* bytes) {
    if (!c || !c->has_volume) return set_error(VPT_ERR_NOT_READY, "no volume");
    if (active) *active = c->active_leaves;
    if (total) *total = c->total_leaves;
    if (gmaj) *gmaj = c->global_majorant;
    if (bytes) *bytes = c->active_leaves * 512 * 4 + c->total_leaves * 8;
    return VPT_OK;
}

int vpt_download_cell_majorants(VptContext* c, float* host) {
    if (!c || !host || !c->has_volume) return set_error(VPT_ERR_NOT_READY, "no volume");
    VPT_CUDA(cudaDeviceSynchronize());
    VPT_CUDA(cudaMemcpy(host, c->d_cell_maj, c->total_leaves * sizeof(float), cudaMemcpyDeviceToHost));
    return VPT_OK;
}

// ------------------------------------------------------------------------------ environment
static int imp_map_layout(int w, int h, VptContextImpl* c) {
    auto next_pow2 = [](uint32_t v) {
        uint32_t p = 1;
        while (p < v) p <<= 1;
        return p;
    };
    uint32_t dx = next_pow2(w);
    uint32_t dy = std::max(next_pow2(h), dx >> 1);
    int levels = 1;
    while ((1u << (levels - 1)) < dx) ++levels;
    if (levels > 16) return set_error(VPT_ERR_INVALID_ARGUMENT, "environment too large");
    c->map_w = dx;
    c->map_h = dy;
    c->num_mips = levels;
    int64_t off = 0;
    for (int l = 0; l < levels; ++l) {
        c->mip_offset[l] = off;
        off += std::max<int64_t>(dx >> l, 1) * std::max<int64_t>(dy >> l, 1);
    }
    c->mip_total = off;
    return VPT_OK;
}

static int finish_environment(VptContext* c) {
    int rc;
    if ((rc = imp_map_layout(c->env_w, c->env_h, c))) return rc;
    if ((rc = dev_alloc(&c->d_mips, c->mip_total))) return rc;
    vpt::build_importance_map(c->d_env, c->env_w, c->env_h, c->map_w, c->map_h, c->num_mips, c->mip_offset, c->d_mips,
                              c->d_integral, 0);
    VPT_CUDA(cudaGetLastError());
    if (c->num_mips == 1) {
        // A 1x1 map: the integral is the single texel.
        VPT_CUDA(cudaMemcpy(c->d_integral, c->d_mips, sizeof(float), cudaMemcpyDeviceToDevice));
    }
    VPT_CUDA(cudaMemcpy(&c->imp_integral, c->d_integral, sizeof(float), cudaMemcpyDeviceToHost));
    return VPT_OK;
}

int vpt_set_environment_rgb(VptContext* c, const float* host_rgb, int32_t w, int32_t h) {
    if (!c || !host_rgb || w <= 0 || h <= 0 || w > 32768 || h > 32768)
        return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_set_environment_rgb: bad arguments");
    std::vector<float4> tex(static_cast<size_t>(w) * h);
    for (size_t i = 0; i < tex.size(); ++i) tex[i] = make_float4(host_rgb[3 * i], host_rgb[3 * i + 1], host_rgb[3 * i + 2], 0.0f);
    int rc;
    if ((rc = dev_alloc(&c->d_env, tex.size()))) return rc;
    VPT_CUDA(cudaMemcpy(c->d_env, tex.data(), tex.size() * sizeof(float4), cudaMemcpyHostToDevice));
    c->env_w = w;
    c->env_h = h;
    return finish_environment(c);
}

int vpt_get_importance_map_info(VptContext* c, int32_t* mw, int32_t* mh, int32_t* nm, int64_t* total, float* integral) {
    if (!c) return set_error(VPT_ERR_INVALID_ARGUMENT, "null context");
    if (mw) *mw = c->map_w;
    if (mh) *mh = c->map_h;
    if (nm) *nm = c->num_mips;
    if (total) *total = c->mip_total;
    if (integral) *integral = c->imp_integral;
    return VPT_OK;
}

int vpt_download_importance_map(VptContext* c, float* host) {
    if (!c || !host) return set_error(VPT_ERR_INVALID_ARGUMENT, "null argument");
    VPT_CUDA(cudaDeviceSynchronize());
    VPT_CUDA(cudaMemcpy(host, c->d_mips, c->mip_total * sizeof(float), cudaMemcpyDeviceToHost));
    return VPT_OK;
}

int vpt_download_environment(VptContext* c, float* host_rgb) {
    if (!c || !host_rgb) return set_error(VPT_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<float4> tex(static_cast<size_t>(c->env_w) * c->env_h);
    VPT_CUDA(cudaDeviceSynchronize());
    VPT_CUDA(cudaMemcpy(tex.data(), c->d_env, tex.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < tex.size(); ++i) {
        host_rgb[3 * i] = tex[i].x;
        host_rgb[3 * i + 1] = tex[i].y;
        host_rgb[3 * i + 2] = tex[i].z;
    }
    return VPT_OK;
}

int vpt_generate_sky(VptContext* c, int32_t w, int32_t h, const float* states, const float* solar, const float* cmf,
                     const float sun_dir[3], int32_t include_solar_disc) {
    if (!c || !states || !solar || !cmf || !sun_dir || w <= 0 || h <= 0 || w > 32768 || h > 32768)
        return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_generate_sky: bad arguments");
    int rc;
    if ((rc = dev_alloc(&c->d_env, static_cast<size_t>(w) * h))) return rc;
    if ((rc = vpt::generate_sky_texture(c->d_env, w, h, states, solar, cmf, sun_dir, include_solar_disc))) return rc;
    c->env_w = w;
    c->env_h = h;
    return finish_environment(c);
}

// ------------------------------------------------------------------------------ frame / launch
int vpt_set_frame_params(VptContext* c, const VptFrameParams* p) {
    if (!c || !p) return set_error(VPT_ERR_INVALID_ARGUMENT, "null argument");
    if (!(p->density_coeff >= 0) || p->phase_kind < 0 || p->phase_kind > 1 || p->majorant_mode < 0 || p->majorant_mode > 1 ||
        p->max_bounces < 0 || !(p->sun_select_prob >= 0 && p->sun_select_prob <= 1) || p->rng_stream_mode < 0 ||
        p->rng_stream_mode > 1 || p->majorant_cell_log2 < 0 || p->majorant_cell_log2 > 10)
        return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_set_frame_params: bad values");
    c->frame = *p;
    c->has_frame = true;
    return VPT_OK;
}

int vpt_set_leaf_staging(VptContext* c, int32_t min_lanes) {
    if (!c || min_lanes < 0 || min_lanes > 32)
        return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_set_leaf_staging: min_lanes must lie in [0, 32]");
    c->leaf_stage_min = min_lanes;
    return VPT_OK;
}

int vpt_set_launch_shape(VptContext* c, int32_t ctas_per_sm, int32_t threads, int32_t park_threshold) {
    if (!c || ctas_per_sm < 0 || threads < 0 || (threads && (threads % 32 || threads > 128)) || park_threshold < 0 ||
        park_threshold > 32)
        return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_set_launch_shape: bad arguments");
    c->ctas_per_sm = ctas_per_sm;
    c->threads = threads;
    c->park_threshold = park_threshold;
    return VPT_OK;
}

}  // extern "C"

namespace vpt {
// LCG jump (multiplier, increment) of `delta` PCG32 draws (O(log delta) advance, Brown 1994).
void lcg_jump(uint64_t delta, uint64_t* mult, uint64_t* plus) {
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
    *mult = acc_mult;
    *plus = acc_plus;
}

// Jump table of a sample-parallel launch: entry i advances a pixel's seed state to the start
// of sample (first + i), i.e. by (first + i) * 2^40 draws.
int upload_sample_jumps(VptContextImpl* c, uint32_t count, cudaStream_t s) {
    if (count > (1u << 20)) return set_error(VPT_ERR_INVALID_ARGUMENT, "at most 2^20 samples per pixel and launch");
    if (c->jump_capacity < count) {
        int rc = dev_alloc(&c->d_jumps, count);
        if (rc) return rc;
        c->jump_capacity = count;
    }
    // Computed on the device, ordered on the launch's stream: no host copy (a copy from pageable
    // memory can block the host until the stream reaches it).
    launch_sample_jump_table_dev(c->d_jumps, c->d_frame, count, s);
    VPT_CUDA(cudaGetLastError());
    return VPT_OK;
}

// Majorant grid of the DDA for the frame's cell size, max-pooled from the 8^3-voxel cells.
static int ensure_majorant_grid(VptContextImpl* c) {
    int shift = c->frame.majorant_cell_log2 < 3 ? 3 : c->frame.majorant_cell_log2;
    if (c->d_maj && c->maj_shift == shift) return VPT_OK;
    int factor = 1 << (shift - 3);
    c->mx = (c->lx + factor - 1) / factor;
    c->my = (c->ly + factor - 1) / factor;
    c->mz = (c->lz + factor - 1) / factor;
    int rc;
    if ((rc = dev_alloc(&c->d_maj, static_cast<size_t>(c->mx) * c->my * c->mz))) return rc;
    pool_majorants(c->d_cell_maj, c->lx, c->ly, c->lz, c->d_maj, c->mx, c->my, c->mz, factor, 0);
    VPT_CUDA(cudaDeviceSynchronize());
    c->maj_shift = shift;
    return VPT_OK;
}

int fill_trace_params(VptContextImpl* c, TraceParams* tp) {
    if ((!c->has_volume && !c->surf) || !c->has_frame)
        return set_error(VPT_ERR_NOT_READY, "volume (or surfaces) or frame parameters missing");
    if (c->has_volume) {
        int rc = ensure_majorant_grid(c);
        if (rc) return rc;
    }
    const VptFrameParams& f = c->frame;
    std::memset(tp, 0, sizeof(*tp));
    tp->volume_enabled = c->has_volume ? 1 : 0;
    if (c->surf) tp->surf = *c->surf;
    Grid& g = tp->grid;
    g.leaf_table = c->d_leaf_table;
    g.leaf_values = c->d_leaf_values;
    g.cell_majorant = c->d_cell_maj;
    g.maj = c->d_maj;
    g.mx = c->mx;
    g.my = c->my;
    g.mz = c->mz;
    g.maj_shift = c->maj_shift;
    g.nx = c->nx;
    g.ny = c->ny;
    g.nz = c->nz;
    g.lx = c->lx;
    g.ly = c->ly;
    g.lz = c->lz;
    g.inv_voxel_size = c->inv_voxel_size;
    for (int a = 0; a < 3; ++a) {
        g.origin[a] = c->origin[a];
        g.bbox_min[a] = c->bbox_min[a];
        g.bbox_max[a] = c->bbox_max[a];
    }
    g.global_majorant = c->global_majorant;
    Env& e = tp->env;
    e.texels = c->d_env;
    e.mips = c->d_mips;
    for (int l = 0; l < 16; ++l) e.mip_offset[l] = c->mip_offset[l];
    e.w = c->env_w;
    e.h = c->env_h;
    e.map_w = c->map_w;
    e.map_h = c->map_h;
    e.num_mips = c->num_mips;
    e.integral = c->imp_integral;
    e.power = f.env_power;
    e.rotation = f.env_rotation;
    tp->env_enabled = f.env_enabled;
    for (int a = 0; a < 3; ++a) {
        tp->sun.dir[a] = f.sun_direction[a];
        tp->sun.irradiance[a] = f.sun_irradiance[a];
        tp->cam_pos[a] = f.cam_position[a];
    }
    for (int a = 0; a < 4; ++a) tp->cam_quat[a] = f.cam_orientation[a];
    tp->sun.select_prob = f.sun_select_prob;
    tp->sun.enabled = f.sun_enabled;
    tp->cam_aspect = f.cam_aspect;
    tp->cam_fovy = f.cam_fovy;
    tp->width = c->width;
    tp->height = c->height;
    tp->density_coeff = f.density_coeff;
    tp->albedo = f.scattering_albedo;
    tp->phase_kind = f.phase_kind;
    tp->phase_param = f.phase_param;
    tp->world_radius = c->world_radius;
    for (int a = 0; a < 3; ++a) {
        tp->world_min[a] = c->world_min[a];
        tp->world_max[a] = c->world_max[a];
    }
    tp->max_bounces = f.max_bounces;
    tp->rr_start = f.rr_start_vertex;
    tp->max_steps = f.max_steps_per_segment;
    tp->shadow_rr = f.shadow_rr_threshold > 0.0f && f.shadow_rr_threshold < 1.0f ? f.shadow_rr_threshold : 0.0f;
    tp->rng = c->d_rng;
    tp->sum_rgb = c->d_sum;
    tp->mean_rgb = c->d_mean;
    tp->work_counter = c->d_work;
    tp->counters = c->d_counters;
    tp->error_flags = c->d_err;
    return VPT_OK;
}

int persistent_grid(VptContextImpl* c, int threads, const void* kernel, size_t smem) {
    int per_sm = c->ctas_per_sm;
    if (per_sm <= 0) {
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem) != cudaSuccess || occ <= 0) occ = 1;
        per_sm = occ;
    }
    return c->num_sms * per_sm;
}
}  // namespace vpt

extern "C" {

static int launch_plain_impl(VptContext* c, void* stream, uint32_t spp, uint32_t* dlog) {
    if (!c || spp == 0) return set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_launch_plain: bad arguments");
    vpt::TraceParams tp;
    int rc = vpt::fill_trace_params(c, &tp);
    if (rc) return rc;
    tp.spp = spp;
    tp.accum_base = c->accum_samples;
    tp.dlog = dlog;
    tp.stream_mode = c->frame.rng_stream_mode;
    tp.stream_base = c->stream_samples;
    tp.park_threshold = c->park_threshold;
    uint64_t npix = static_cast<uint64_t>(c->width) * c->height;
    if (npix * spp >= (1ull << 31)) return set_error(VPT_ERR_INVALID_ARGUMENT, "too many samples in one launch");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (tp.stream_mode == 1) {
        int rc2 = vpt::upload_sample_jumps(c, spp, s);
        if (rc2) return rc2;
        tp.sample_jumps = c->d_jumps;
    }
    VPT_CUDA(cudaMemsetAsync(c->d_work, 0, sizeof(unsigned int), s));
    bool grid_maj = c->frame.majorant_mode == 1 && c->has_volume;
    size_t smem = 0;
    if (grid_maj && c->mx * c->my * c->mz <= vpt::kMajSmemCells) {
        tp.maj_in_smem = 1;
        smem = static_cast<size_t>(c->mx) * c->my * c->mz * sizeof(float);
    }
    // Leaf staging: majorant-grid tracker on sample-parallel streams (and its logged form).
    const bool stage = c->leaf_stage_min > 0 && grid_maj && (dlog != nullptr || tp.stream_mode == 1) && !c->surf;
    tp.leaf_stage_min = stage ? c->leaf_stage_min : 0;
    // One 896-thread CTA per SM for the production plain tracer on sample-parallel streams; the
    // other forms (and leaf staging, whose per-warp buffers would exceed the default dynamic
    // shared-memory limit at 28 warps) run CTAs of 128.
    const bool sp_plain = dlog == nullptr && tp.stream_mode == 1 && !c->surf && c->tracker != 1 && !stage;
    const int threads = c->threads > 0 ? c->threads : (sp_plain ? vpt::kPlainSampleParallelThreads : 128);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &capture) != cudaSuccess) capture = cudaStreamCaptureStatusActive;
    if (c->surf) {
        // Scenes with triangles: the surface form of the persistent tracker.
        const void* kernel = vpt::surface_kernel_ptr(grid_maj, dlog != nullptr);
        int ctas = vpt::persistent_grid(c, threads, kernel, smem);
        vpt::launch_surface(tp, grid_maj, ctas, threads, smem, s);
    } else if (c->tracker == 1 && capture == cudaStreamCaptureStatusNone) {
        // Wavefront tracer: its passes are issued from the host until every slot retired (not
        // capturable; a stream being captured gets the persistent megakernel below).
        const uint64_t items = tp.stream_mode == 1 ? npix * spp : npix;
        const uint64_t per_sm = c->wf_slots_per_sm > 0 ? static_cast<uint64_t>(c->wf_slots_per_sm) : 3072u;
        const uint32_t slots = static_cast<uint32_t>(std::min<uint64_t>(items, per_sm * c->num_sms));
        int rc3 = vpt::wf_ensure(c, slots);
        if (rc3) return rc3;
        rc3 = vpt::wf_run(c, tp, grid_maj, smem, s);
        if (rc3) return rc3;
    } else {
        const size_t launch_smem = vpt::plain_smem_bytes(smem, stage, threads);
        const void* kernel = vpt::plain_kernel_ptr(grid_maj, dlog != nullptr, tp.stream_mode == 1, stage);
        int ctas = vpt::persistent_grid(c, threads, kernel, launch_smem);
        vpt::launch_plain(tp, grid_maj, ctas, threads, launch_smem, s);
    }
    if (tp.stream_mode == 1)
        vpt::launch_finalize_mean_dev(c->d_sum, c->d_mean, static_cast<uint32_t>(3 * npix), c->d_frame, spp, s);
    vpt::launch_frame_update(c->d_frame, spp, false, spp, s);
    c->accum_samples += spp;
    c->stream_samples += spp;
    VPT_CUDA(cudaGetLastError());
    return VPT_OK;
}

int vpt_launch_plain(VptContext* c, void* stream, uint32_t spp) { return launch_plain_impl(c, stream, spp, nullptr); }

int vpt_launch_plain_logged(VptContext* c, void* stream, uint32_t spp, uint32_t* dev_log) {
    if (!dev_log) return set_error(VPT_ERR_INVALID_ARGUMENT, "null log buffer");
    return launch_plain_impl(c, stream, spp, dev_log);
}

int vpt_download_sum(VptContext* c, double* host, uint32_t* n) {
    if (!c || !host) return set_error(VPT_ERR_INVALID_ARGUMENT, "null argument");
    int64_t npix = static_cast<int64_t>(c->width) * c->height;
    VPT_CUDA(cudaDeviceSynchronize());
    VPT_CUDA(cudaMemcpy(host, c->d_sum, 3 * npix * sizeof(double), cudaMemcpyDeviceToHost));
    if (n) {
        uint32_t frame[2];
        VPT_CUDA(cudaMemcpy(frame, c->d_frame, sizeof(frame), cudaMemcpyDeviceToHost));
        *n = frame[1];  // advanced on the device, also by replays of captured launches
    }
    return VPT_OK;
}

int vpt_download_mean(VptContext* c, float* host) {
    if (!c || !host) return set_error(VPT_ERR_INVALID_ARGUMENT, "null argument");
    int64_t npix = static_cast<int64_t>(c->width) * c->height;
    VPT_CUDA(cudaDeviceSynchronize());
    VPT_CUDA(cudaMemcpy(host, c->d_mean, 3 * npix * sizeof(float), cudaMemcpyDeviceToHost));
    return VPT_OK;
}

int vpt_get_accum_device_ptrs(VptContext* c, double** sum, float** mean) {
    if (!c) return set_error(VPT_ERR_INVALID_ARGUMENT, "null context");
    if (sum) *sum = c->d_sum;
    if (mean) *mean = c->d_mean;
    return VPT_OK;
}

int vpt_get_counters(VptContext* c, uint64_t* lookups, uint64_t* vertices, uint64_t* samples, uint64_t* cells) {
    if (!c) return set_error(VPT_ERR_INVALID_ARGUMENT, "null context");
    unsigned long long h[8];
    VPT_CUDA(cudaDeviceSynchronize());
    VPT_CUDA(cudaMemcpy(h, c->d_counters, sizeof(h), cudaMemcpyDeviceToHost));
    if (lookups) *lookups = h[0];
    if (vertices) *vertices = h[1];
    if (samples) *samples = h[2];
    if (cells) *cells = h[3];
    return VPT_OK;
}

int vpt_reset_counters(VptContext* c) {
    if (!c) return set_error(VPT_ERR_INVALID_ARGUMENT, "null context");
    VPT_CUDA(cudaMemset(c->d_counters, 0, 8 * sizeof(unsigned long long)));
    VPT_CUDA(cudaMemset(c->d_err, 0, sizeof(unsigned int)));
    return VPT_OK;
}

uint32_t vpt_get_device_errors(VptContext* c) {
    if (!c) return 0;
    unsigned int e = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) return 0xffffffffu;
    if (cudaMemcpy(&e, c->d_err, sizeof(e), cudaMemcpyDeviceToHost) != cudaSuccess) return 0xffffffffu;
    return e;
}

int vpt_synchronize(VptContext* c, void* stream) {
    (void)c;
    VPT_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    return VPT_OK;
}

}  // extern "C"

namespace vpt {

// Device side of vpt_set_volume_nanovdb: the flattened leaves (slot order), their table over the
// leaf-aligned extent starting at index `lo`, and the grid's map and boxes. Cell majorants use
// the same apron as the dense build; the global majorant scans [index_min, index_max) of the
// grid's index box (renderer/renderer_scene.cpp:498-509).
int upload_sparse_grid(VptContextImpl* c, const std::vector<int32_t>& table, int32_t lx, int32_t ly, int32_t lz,
                       const std::vector<int32_t>& origins, const float* values, int64_t slots, const int32_t lo[3],
                       const VptNanoVdbInfo& info) {
    const int64_t cells = static_cast<int64_t>(lx) * ly * lz;
    dev_free(&c->d_dense);
    c->has_volume = false;
    int32_t* d_origins = nullptr;
    int rc;
    if ((rc = dev_alloc(&c->d_cell_maj, cells)) || (rc = dev_alloc(&c->d_leaf_table, cells)) ||
        (rc = dev_alloc(&c->d_leaf_values, std::max<int64_t>(slots, 1) * 512)) ||
        (rc = dev_alloc(&d_origins, std::max<int64_t>(slots, 1) * 3)))
        return rc;
    VPT_CUDA(cudaMemcpy(c->d_leaf_table, table.data(), cells * sizeof(int32_t), cudaMemcpyHostToDevice));
    if (slots > 0) {
        VPT_CUDA(cudaMemcpy(c->d_leaf_values, values, slots * 512 * sizeof(float), cudaMemcpyHostToDevice));
        VPT_CUDA(cudaMemcpy(d_origins, origins.data(), slots * 3 * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    c->lx = lx;
    c->ly = ly;
    c->lz = lz;
    c->nx = 8 * lx;
    c->ny = 8 * ly;
    c->nz = 8 * lz;
    vpt::sparse_leaf_stats(c->d_leaf_table, c->d_leaf_values, lx, ly, lz, c->d_cell_maj, 0);
    int32_t box_lo[3], box_hi[3];
    for (int a = 0; a < 3; ++a) {
        box_lo[a] = info.index_min[a] - lo[a];
        box_hi[a] = info.index_max[a] - lo[a];
    }
    vpt::leaf_box_max(c->d_leaf_values, d_origins, slots, box_lo, box_hi, c->d_scratch_u32, 0);
    cudaError_t e = cudaGetLastError();
    unsigned int gmax_bits = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&gmax_bits, c->d_scratch_u32, sizeof(unsigned int), cudaMemcpyDeviceToHost);
    dev_free(&d_origins);
    if (e != cudaSuccess) return set_error(VPT_ERR_CUDA, std::string("vpt_set_volume_nanovdb: ") + cudaGetErrorString(e));
    std::memcpy(&c->global_majorant, &gmax_bits, sizeof(float));
    c->active_leaves = slots;
    c->total_leaves = cells;
    // Lookups map world p to index (p - origin) * inv_voxel_size, origin being the world position
    // of the extent's first voxel; for an extent starting at index 0 that is the grid's own
    // float map (NanoVDB.h:2029-2032, applyInverseMapF).
    c->voxel_size = info.map_mat_f[0];
    c->inv_voxel_size = info.map_inv_mat_f[0];
    for (int a = 0; a < 3; ++a) {
        c->origin[a] = static_cast<float>(info.map_vec_d[a] + static_cast<double>(lo[a]) * info.map_mat_d[4 * a]);
        c->bbox_min[a] = static_cast<float>(info.world_min[a]);
        c->bbox_max[a] = static_cast<float>(info.world_max[a]);
    }
    c->has_volume = true;
    c->update_world_box();
    c->maj_shift = 0;  // the pooled majorant grid is rebuilt at the next launch
    VPT_CUDA(cudaDeviceSynchronize());
    return VPT_OK;
}

}  // namespace vpt
