// Allocation-free launch of the plain tracer (vpt_launch_plain_noalloc).
//
// Some callers cannot call cudaMalloc: a host renderer whose device memory is owned by its own
// pool allocator, or code running where allocation is not allowed. For them this entry point
// takes every input and output as caller-owned device pointers and keeps the launch's scratch
// memory — the work counter, the work counters, the error word and the per-launch table of
// RNG jump constants — in one file-scope __device__ array of fixed size (kScratchBytes), which
// every GPU that loads the library holds until exit. It makes no allocation: no cudaMalloc,
// cudaFree or allocating library routine, and no host heap buffer either (the jump table is
// computed on the device).
//
// The array is shared by all calls: calls that overlap on the GPU (different streams, or
// threads) race on it. Its address is looked up with cudaGetSymbolAddress on the first call
// made with a device current, so make that first call before any stream capture. The address
// belongs to the context it was looked up in: when the current context of the device changes
// (for instance after cudaDeviceReset), the next call looks it up again.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/rtc8_vpt.h"
#include "vpt_ctx.h"
#include "vpt_tracer.cuh"

namespace vpt {
namespace {

constexpr uint32_t kNoAllocMaxSpp = VPT_NOALLOC_MAX_SPP;
constexpr size_t kScratchHeader = 256;  // [0] work counter, [8..72) counters, [72] error word
constexpr size_t kScratchBytes = kScratchHeader + kNoAllocMaxSpp * sizeof(ulonglong2);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
struct ScratchSlot {
    unsigned long long context_id;  // unique id of the context the address was looked up in
    unsigned char* ptr;
};
ScratchSlot g_scratch[kMaxDevices] = {};

// Driver entry points reached through the runtime (the library does not link libcuda).
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Unique id of the calling thread's current context; false when none is current yet.
bool current_context_id(unsigned long long* id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
            qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
            return false;
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(a);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(b);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return g_ctx_get_id(ctx, id) == CUDA_SUCCESS;
}

// Device address of the scratch array in the current device's current context (looked up once
// per device and context).
int scratch_address(unsigned char** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return ctx_set_error(VPT_ERR_CUDA, "vpt_launch_plain_noalloc: no usable current device");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    ScratchSlot& slot = g_scratch[dev];
    unsigned long long id = 0;
    const bool have_id = current_context_id(&id);
    if (!slot.ptr || !have_id || slot.context_id != id) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // makes the primary context current
        if (e != cudaSuccess || !p)
            return ctx_set_error(VPT_ERR_CUDA, "vpt_launch_plain_noalloc: cudaGetSymbolAddress of the scratch failed");
        if (!current_context_id(&id))
            return ctx_set_error(VPT_ERR_CUDA, "vpt_launch_plain_noalloc: no current context after the set-up");
        slot.ptr = static_cast<unsigned char*>(p);
        slot.context_id = id;
    }
    *out = slot.ptr;
    return VPT_OK;
}

}  // namespace
}  // namespace vpt

extern "C" int vpt_launch_plain_noalloc(const VptNoAllocTrace* a, void* stream) {
    using namespace vpt;
    if (!a || !a->leaf_table || !a->leaf_values || !a->majorants || !a->env_texels || !a->imp_mips || !a->rng ||
        !a->sum_rgb || !a->mean_rgb)
        return ctx_set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_launch_plain_noalloc: null pointer");
    const VptFrameParams& f = a->frame;
    if (a->width <= 0 || a->height <= 0 || a->nx <= 1 || a->ny <= 1 || a->nz <= 1 || !(a->voxel_size > 0) ||
        a->env_w <= 0 || a->env_h <= 0 || a->map_w <= 0 || a->map_h <= 0 || a->num_mips <= 0 || a->num_mips > 16)
        return ctx_set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_launch_plain_noalloc: bad sizes");
    if (a->spp == 0 || a->spp > kNoAllocMaxSpp)
        return ctx_set_error(VPT_ERR_INVALID_ARGUMENT,
                             "vpt_launch_plain_noalloc: spp must be in [1, VPT_NOALLOC_MAX_SPP] (4096)");
    uint64_t npix = static_cast<uint64_t>(a->width) * a->height;
    if (npix * a->spp >= (1ull << 31))
        return ctx_set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_launch_plain_noalloc: too many samples in one launch");
    if (!(f.density_coeff >= 0) || f.phase_kind < 0 || f.phase_kind > 1 || f.majorant_mode < 0 || f.majorant_mode > 1 ||
        f.max_bounces < 0 || f.rng_stream_mode < 0 || f.rng_stream_mode > 1 || f.majorant_cell_log2 < 0 ||
        f.majorant_cell_log2 > 10 || !(f.sun_select_prob >= 0 && f.sun_select_prob <= 1))
        return ctx_set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_launch_plain_noalloc: bad frame parameters");
    const int shift = f.majorant_cell_log2 < 3 ? 3 : f.majorant_cell_log2;
    const int cell = 1 << shift;
    if (a->mx != (a->nx + cell - 1) / cell || a->my != (a->ny + cell - 1) / cell || a->mz != (a->nz + cell - 1) / cell)
        return ctx_set_error(VPT_ERR_INVALID_ARGUMENT,
                             "vpt_launch_plain_noalloc: majorant grid dims do not match 2^majorant_cell_log2 cells");

    unsigned char* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    TraceParams tp;
    std::memset(&tp, 0, sizeof(tp));
    Grid& g = tp.grid;
    g.leaf_table = a->leaf_table;
    g.leaf_values = a->leaf_values;
    g.cell_majorant = a->majorants;
    g.maj = a->majorants;
    g.mx = a->mx;
    g.my = a->my;
    g.mz = a->mz;
    g.maj_shift = shift;
    g.nx = a->nx;
    g.ny = a->ny;
    g.nz = a->nz;
    g.lx = (a->nx + 7) / 8;
    g.ly = (a->ny + 7) / 8;
    g.lz = (a->nz + 7) / 8;
    g.inv_voxel_size = static_cast<float>(1.0 / static_cast<double>(a->voxel_size));
    int n[3] = {a->nx, a->ny, a->nz};
    float r2 = 0.0f;
    for (int i = 0; i < 3; ++i) {
        g.origin[i] = a->origin[i];
        g.bbox_min[i] = a->origin[i];
        g.bbox_max[i] = static_cast<float>(a->origin[i] + static_cast<double>(n[i]) * a->voxel_size);
        float center = (g.bbox_min[i] + g.bbox_max[i]) * 0.5f;
        float d = g.bbox_max[i] - center;
        r2 += d * d;
    }
    g.global_majorant = a->global_majorant;
    Env& e = tp.env;
    e.texels = reinterpret_cast<const float4*>(a->env_texels);
    e.mips = a->imp_mips;
    int64_t off = 0;
    for (int l = 0; l < a->num_mips; ++l) {
        e.mip_offset[l] = off;
        off += static_cast<int64_t>(std::max(a->map_w >> l, 1)) * std::max(a->map_h >> l, 1);
    }
    e.w = a->env_w;
    e.h = a->env_h;
    e.map_w = a->map_w;
    e.map_h = a->map_h;
    e.num_mips = a->num_mips;
    e.integral = a->imp_integral;
    e.power = f.env_power;
    e.rotation = f.env_rotation;
    tp.env_enabled = f.env_enabled;
    for (int i = 0; i < 3; ++i) {
        tp.sun.dir[i] = f.sun_direction[i];
        tp.sun.irradiance[i] = f.sun_irradiance[i];
        tp.cam_pos[i] = f.cam_position[i];
    }
    for (int i = 0; i < 4; ++i) tp.cam_quat[i] = f.cam_orientation[i];
    tp.sun.select_prob = f.sun_select_prob;
    tp.sun.enabled = f.sun_enabled;
    tp.cam_aspect = f.cam_aspect;
    tp.cam_fovy = f.cam_fovy;
    tp.width = a->width;
    tp.height = a->height;
    tp.density_coeff = f.density_coeff;
    tp.albedo = f.scattering_albedo;
    tp.phase_kind = f.phase_kind;
    tp.phase_param = f.phase_param;
    tp.world_radius = std::sqrt(r2);
    tp.max_bounces = f.max_bounces;
    tp.rr_start = f.rr_start_vertex;
    tp.max_steps = f.max_steps_per_segment;
    tp.shadow_rr = f.shadow_rr_threshold > 0.0f && f.shadow_rr_threshold < 1.0f ? f.shadow_rr_threshold : 0.0f;
    tp.spp = a->spp;
    tp.accum_base = a->accum_base;
    tp.stream_mode = f.rng_stream_mode;
    tp.stream_base = a->stream_base;
    tp.rng = a->rng;
    tp.sum_rgb = a->sum_rgb;
    tp.mean_rgb = a->mean_rgb;
    tp.work_counter = reinterpret_cast<unsigned int*>(scratch);
    tp.counters = reinterpret_cast<unsigned long long*>(scratch + 8);
    // Error bits go to the caller's word when one is given (ORed in; the caller clears it).
    tp.error_flags = a->device_errors ? a->device_errors : reinterpret_cast<unsigned int*>(scratch + 72);
    ulonglong2* jumps = reinterpret_cast<ulonglong2*>(scratch + kScratchHeader);
    tp.sample_jumps = jumps;

    // The scratch keeps the previous call's contents: clear what must start at zero.
    if (cudaMemsetAsync(scratch, 0, kScratchHeader, s) != cudaSuccess)
        return ctx_set_error(VPT_ERR_CUDA, "vpt_launch_plain_noalloc: clearing the scratch failed");
    if (tp.stream_mode == 1) launch_sample_jump_table(jumps, a->stream_base, a->spp, s);

    const int threads = 128;
    const bool grid_maj = f.majorant_mode == 1;
    size_t smem = 0;
    if (grid_maj && a->mx * a->my * a->mz <= kMajSmemCells) {
        tp.maj_in_smem = 1;
        smem = static_cast<size_t>(a->mx) * a->my * a->mz * sizeof(float);
    }
    int dev = 0, sms = 0, occ = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return ctx_set_error(VPT_ERR_CUDA, "vpt_launch_plain_noalloc: device query failed");
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, plain_kernel_ptr(grid_maj, false, tp.stream_mode == 1, false), threads, smem) != cudaSuccess ||
        occ <= 0)
        occ = 1;
    launch_plain(tp, grid_maj, sms * occ, threads, smem, s);
    if (tp.stream_mode == 1)
        launch_finalize_mean(a->sum_rgb, a->mean_rgb, static_cast<uint32_t>(3 * npix), a->accum_base + a->spp, s);
    if (cudaGetLastError() != cudaSuccess) return ctx_set_error(VPT_ERR_CUDA, "vpt_launch_plain_noalloc: launch failed");
    return VPT_OK;
}
