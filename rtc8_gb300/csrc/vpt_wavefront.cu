// Wavefront form of the plain volumetric path tracer (the reference's pathTrace ray-generation
// program, renderer/gpu_kernels/optix_pathtracing_kernels.cu:31-434 with withNRC = false).
//
// The work of a launch is split over two kernels that alternate in passes, with every path's
// state kept per slot in structure-of-arrays device buffers (coalesced by slot index):
//   * wf_event_kernel, one thread per queued slot: everything but tracking — fetching a work
//     item (path regeneration), the camera ray, segment set-up and clipping, the in-medium
//     vertex (Russian roulette, NEE light selection and sampling), the NEE contribution and
//     phase sampling, the environment hit, the end of a sample and its accumulation. It runs a
//     slot's state machine until the slot needs a tracked segment (queued for tracking) or has
//     no work left (retired).
//   * wf_track_kernel, persistent: each lane takes a segment from the tracking queue, runs
//     delta tracking (primary segments) or ratio tracking (shadow segments) through the global
//     majorant or the majorant-grid DDA, and takes the next queued segment as soon as its own
//     ends, so the lanes of a warp stay busy with density lookups instead of waiting for each
//     other's events. A segment gets at most `pass_steps` lookups per pass; a longer one is
//     suspended (its DDA state saved) and continues in the next pass, so no pass waits on the
//     longest segment of the image.
// Queues are compacted with warp-aggregated atomics; the host issues passes until the tracking
// queue stays empty after an event pass. Per path the random numbers are drawn in exactly the
// order of the persistent megakernel (vpt_tracer.cu), so both produce the same decisions.
// This unit is compiled without multiply-add contraction, like the megakernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "vpt_ctx.h"
#include "vpt_tracer.cuh"

namespace vpt {
namespace {

enum : uint32_t {
    WS_FETCH = 0,
    WS_CAMERA,
    WS_SEGMENT,
    WS_STEP,       // waiting for (or in) tracking
    WS_VERTEX,     // primary collision at seg.t
    WS_NEE_DONE,   // shadow segment finished (vis)
    WS_ESCAPE,
    WS_END_SAMPLE,
    WS_DONE,
};

enum : uint32_t {
    WE_ESCAPE = 1,
    WE_RR = 2,
    WE_PDF_ZERO = 3,
    WE_MAX_BOUNCES = 4,
    WE_STEP_CAP = 5,
};

constexpr uint32_t kHardStepCap = 1u << 24;
constexpr uint32_t kHardVertexCap = 1u << 16;

// flags word of a slot
constexpr uint32_t kFlagShadow = 1u << 16;   // the queued segment is a shadow (NEE) segment
constexpr uint32_t kFlagPickSun = 1u << 17;  // the NEE sample picked the sun
constexpr uint32_t kFlagResume = 1u << 18;   // the segment was suspended: DDA state saved
__device__ __forceinline__ uint32_t st_of(uint32_t f) { return f & 0xFFu; }
__device__ __forceinline__ uint32_t end_of(uint32_t f) { return (f >> 8) & 0xFFu; }
__device__ __forceinline__ uint32_t make_flags(uint32_t st, uint32_t end, uint32_t bits) {
    return st | (end << 8) | bits;
}

// Majorant-grid DDA (the megakernel's definition, vpt_tracer.cu).
struct Dda {
    int cell[3];
    int step[3];
    float tnext[3], tdelta[3];
};

__device__ __forceinline__ void dda_init(const Grid& g, V3 eye, V3 dir, float t, Dda* d) {
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

// step and tdelta of a resumed segment (the values dda_init computed for it).
__device__ __forceinline__ void dda_steps(const Grid& g, V3 dir, Dda* d) {
    float dd[3] = {dir.x * g.inv_voxel_size, dir.y * g.inv_voxel_size, dir.z * g.inv_voxel_size};
    const float size = static_cast<float>(1 << g.maj_shift);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (dd[a] > 0) {
            d->step[a] = 1;
            d->tdelta[a] = size / dd[a];
        } else if (dd[a] < 0) {
            d->step[a] = -1;
            d->tdelta[a] = -size / dd[a];
        } else {
            d->step[a] = 0;
            d->tdelta[a] = INFINITY;
        }
    }
}

__device__ __forceinline__ float cell_maj(const float* maj, const Grid& g, const Dda& d) {
    return maj[(d.cell[0] * g.my + d.cell[1]) * g.mz + d.cell[2]];
}

// Appends `slot` to a queue for every lane with `push` set; all 32 lanes of the warp call it.
__device__ __forceinline__ void warp_push(bool push, uint32_t slot, uint32_t* queue, uint32_t* count) {
    const uint32_t m = __ballot_sync(0xffffffffu, push);
    if (m == 0) return;
    const uint32_t lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (static_cast<int>(lane) == leader) base = atomicAdd(count, static_cast<uint32_t>(__popc(m)));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (push) queue[base + __popc(m & ((1u << lane) - 1u))] = slot;
}

// ------------------------------------------------------------------------------ event kernel
// One thread per queued slot (first pass: every slot). Runs the slot's state machine until it
// needs tracking or retires.
__global__ void __launch_bounds__(128) wf_event_kernel(const TraceParams P, const WfBuffers W, int first_pass,
                                                       uint32_t in_q, uint32_t out_q) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // The counters the following tracking pass fills.
        W.count[2 + (out_q ^ 1)] = 0;  // next event queue
        W.count[(out_q ^ 1)] = 0;      // next tracking queue (suspended segments)
        W.count[4] = 0;                // tracking fetch counter
    }
    const Grid& g = P.grid;
    const uint32_t num_pixels = static_cast<uint32_t>(P.width) * static_cast<uint32_t>(P.height);
    const V3 bmin = v3(g.bbox_min[0], g.bbox_min[1], g.bbox_min[2]);
    const V3 bmax = v3(g.bbox_max[0], g.bbox_max[1], g.bbox_max[2]);
    const uint32_t n = first_pass ? W.slots : W.count[2 + in_q];
    unsigned long long n_vertices = 0, n_samples = 0;
    unsigned int err = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        const uint32_t slot = valid ? (first_pass ? i : W.event_queue[in_q * W.slots + i]) : 0;
        bool push_track = false;
        if (valid) {
            uint32_t flags = first_pass ? static_cast<uint32_t>(WS_FETCH) : W.flags[slot];
            uint32_t st = st_of(flags), end_code = end_of(flags);
            bool pick_sun = flags & kFlagPickSun;
            Pcg32 rng{W.rng[slot]};
            uint32_t pixel = W.pixel[slot], sample = W.sample[slot], path_length = W.path_length[slot];
            float4 a = W.org[slot], b = W.dir[slot], c = W.tp[slot], d = W.contrib[slot], e = W.emit[slot];
            V3 origin = v3(a.x, a.y, a.z), dir = v3(b.x, b.y, b.z);
            float dir_pdf = a.w, init_importance = b.w;
            RGB throughput = rgb(c.x, c.y, c.z), contribution = rgb(d.x, d.y, d.z), emittance = rgb(e.x, e.y, e.z);
            float area_pdf = c.w, vis = d.w;
            uint2 rec = W.rec[slot];
            const float4 s0 = W.seg0[slot], s1 = W.seg1[slot];
            float t = s0.w;
            V3 light_dir = -v3(s1.x, s1.y, s1.z);  // a shadow segment runs towards the vertex
            double sum_r = 0, sum_g = 0, sum_b = 0;
            RGB mean = rgb(0, 0, 0);
            if (P.stream_mode != 1 && !first_pass) {
                sum_r = W.sum[3 * slot];
                sum_g = W.sum[3 * slot + 1];
                sum_b = W.sum[3 * slot + 2];
                const float4 m = W.mean[slot];
                mean = rgb(m.x, m.y, m.z);
            }
            V3 seg_eye = origin, seg_dir = dir;
            float t1 = 0.0f;
            while (st != WS_STEP && st != WS_DONE) {
                switch (st) {
                case WS_FETCH: {
                    const uint32_t need = __activemask();
                    const int leader = __ffs(need) - 1;
                    const uint32_t lane = threadIdx.x & 31;
                    uint32_t wb = 0;
                    if (static_cast<int>(lane) == leader) wb = atomicAdd(P.work_counter, __popc(need));
                    wb = __shfl_sync(need, wb, leader);
                    const uint32_t item = wb + __popc(need & ((1u << lane) - 1u));
                    if (P.stream_mode == 1) {
                        if (item >= num_pixels * P.spp) {
                            st = WS_DONE;
                            break;
                        }
                        pixel = item % num_pixels;
                        sample = item / num_pixels;
                        const ulonglong2 jump = P.sample_jumps[sample];
                        rng.state = jump.x * P.rng[pixel] + jump.y;
                        st = WS_CAMERA;
                        break;
                    }
                    if (item >= num_pixels) {
                        st = WS_DONE;
                        break;
                    }
                    pixel = item;
                    rng.state = P.rng[pixel];
                    sum_r = sum_g = sum_b = 0;
                    if (P.accum_base > 0) {
                        mean = rgb(P.mean_rgb[3 * pixel], P.mean_rgb[3 * pixel + 1], P.mean_rgb[3 * pixel + 2]);
                    } else {
                        mean = rgb(0, 0, 0);
                    }
                    sample = 0;
                    st = WS_CAMERA;
                    break;
                }
                case WS_CAMERA: {
                    // optix_pathtracing_kernels.cu:43-55, 76-81.
                    const uint32_t img_w = static_cast<uint32_t>(P.width), img_h = static_cast<uint32_t>(P.height);
                    uint32_t px = pixel % img_w;
                    uint32_t py = pixel / img_w;
                    float ux = rng.uniform();
                    float fx = (px + ux) / static_cast<float>(img_w);
                    float uy = rng.uniform();
                    float fy = (py + uy) / static_cast<float>(img_h);
                    float vh = 2 * tanf(P.cam_fovy * 0.5f);
                    float vw = P.cam_aspect * vh;
                    float sensor_area = vw * vh;
                    origin = v3(P.cam_pos[0], P.cam_pos[1], P.cam_pos[2]);
                    V3 local = normalize(v3(vw * (-0.5f + fx), vh * (0.5f - fy), -1));
                    dir = normalize(mul(quat_to_m3(P.cam_quat[0], P.cam_quat[1], P.cam_quat[2], P.cam_quat[3]), local));
                    float az = fabsf(local.z);
                    dir_pdf = 1 / (az * az * az * sensor_area);
                    float inv = 1.0f / dir_pdf;
                    throughput = rgb(1, 1, 1) * inv;
                    init_importance = luminance(throughput);
                    contribution = rgb(0, 0, 0);
                    path_length = 0;
                    end_code = 0;
                    rec = make_uint2(0, 0);
                    st = WS_SEGMENT;
                    break;
                }
                case WS_SEGMENT: {
                    ++path_length;
                    ++n_vertices;
                    if (path_length > kHardVertexCap) {
                        end_code = WE_MAX_BOUNCES;
                        st = WS_END_SAMPLE;
                        break;
                    }
                    float ta, tb;
                    if (clip_ray(bmin, bmax, origin, dir, 0.0f, 1e10f, &ta, &tb)) {
                        seg_eye = origin;
                        seg_dir = dir;
                        t = fmaxf(0.0f, ta);
                        t1 = tb;
                        flags = 0;
                        st = WS_STEP;
                    } else {
                        st = WS_ESCAPE;
                    }
                    break;
                }
                case WS_VERTEX: {
                    // In-medium vertex (:176-182), Russian roulette (:254-268, 332), NEE set-up
                    // (renderer_kernel_common.h:297-358).
                    origin = origin + t * dir;
                    float continue_prob = 1.0f;
                    if (static_cast<int32_t>(path_length) >= P.rr_start) {
                        continue_prob = fminf(luminance(throughput) / init_importance, 1.0f);
                        if (rng.uniform() >= continue_prob) {
                            end_code = WE_RR;
                            st = WS_END_SAMPLE;
                            break;
                        }
                    }
                    throughput = rdiv(throughput, continue_prob);
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
                        st = WS_NEE_DONE;  // vis = 0: no contribution
                        break;
                    }
                    vis = 1.0f;
                    float trace_len = 2 * P.world_radius;
                    seg_dir = -light_dir;
                    seg_eye = origin + trace_len * -seg_dir;
                    float ta, tb;
                    if (clip_ray(bmin, bmax, seg_eye, seg_dir, 0.0f, trace_len, &ta, &tb)) {
                        t = fmaxf(0.0f, ta);
                        t1 = tb;
                        flags = kFlagShadow;
                        st = WS_STEP;
                    } else {
                        st = WS_NEE_DONE;
                    }
                    break;
                }
                case WS_NEE_DONE: {
                    // renderer_kernel_common.h:385-402, then phase sampling (:341-356).
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
                            float lp_cos = dot(sdir, -light_dir);
                            float bsdf_pdf = pf * lp_cos / 1.0f;
                            if (!isfinite(bsdf_pdf)) bsdf_pdf = 0.0f;
                            float light_pdf = area_pdf;
                            float mis = (light_pdf * light_pdf) / ((bsdf_pdf * bsdf_pdf) + (light_pdf * light_pdf));
                            RGB le = rdiv(emittance, kPi);
                            float gterm = lp_cos * 1.0f / 1.0f;
                            nee = fs * le * (vis * mis * gterm / area_pdf);
                        }
                        contribution = contribution + throughput * nee;
                    }
                    if (P.max_bounces > 0 && static_cast<int32_t>(path_length) >= P.max_bounces) {
                        end_code = WE_MAX_BOUNCES;
                        st = WS_END_SAMPLE;
                        break;
                    }
                    Frame fr = make_frame(-dir);
                    float u0 = rng.uniform();
                    float u1 = rng.uniform();
                    V3 local;
                    float pdf = phase_sample(P.phase_kind, P.phase_param, u0, u1, &local);
                    if (pdf == 0.0f) {
                        end_code = WE_PDF_ZERO;
                        st = WS_END_SAMPLE;
                        break;
                    }
                    RGB fs = rgb(P.albedo, P.albedo, P.albedo) * pdf;
                    dir = from_local(fr, local);
                    RGB local_tp = fs * (fabsf(1.0f) / pdf);
                    throughput = throughput * local_tp;
                    dir_pdf = pdf;
                    st = WS_SEGMENT;
                    break;
                }
                case WS_ESCAPE: {
                    // optix_pathtracing_kernels.cu:130-174.
                    if (P.env_enabled) {
                        float hyp_pdf;
                        RGB radiance = env_evaluate(P.env, dir, &hyp_pdf);
                        float mis = 1.0f;
                        if (path_length > 1) {
                            float light_pdf = (P.sun.enabled ? (1.0f - P.sun.select_prob) : 1.0f) * hyp_pdf;
                            float bsdf_pdf = dir_pdf;
                            mis = (bsdf_pdf * bsdf_pdf) / ((bsdf_pdf * bsdf_pdf) + (light_pdf * light_pdf));
                        }
                        contribution = contribution + throughput * (radiance * mis);
                    }
                    end_code = WE_ESCAPE;
                    st = WS_END_SAMPLE;
                    break;
                }
                case WS_END_SAMPLE: {
                    // optix_pathtracing_kernels.cu:413-432 (non-finite samples are dropped).
                    ++n_samples;
                    if (P.dlog) {
                        uint4 r4 = make_uint4(path_length, rec.x, rec.y, end_code);
                        reinterpret_cast<uint4*>(P.dlog)[static_cast<uint64_t>(pixel) * P.spp + sample] = r4;
                    }
                    if (P.stream_mode == 1) {
                        if (all_nonneg_finite(contribution)) {
                            atomicAdd(P.sum_rgb + 3 * pixel, static_cast<double>(contribution.r));
                            atomicAdd(P.sum_rgb + 3 * pixel + 1, static_cast<double>(contribution.g));
                            atomicAdd(P.sum_rgb + 3 * pixel + 2, static_cast<double>(contribution.b));
                        } else {
                            err |= VPT_DEVERR_NONFINITE;
                        }
                        st = WS_FETCH;
                        break;
                    }
                    if (all_nonneg_finite(contribution)) {
                        sum_r += contribution.r;
                        sum_g += contribution.g;
                        sum_b += contribution.b;
                        uint32_t nacc = P.accum_base + sample;
                        RGB prev = nacc > 0 ? mean : rgb(0, 0, 0);
                        float w = 1.0f / (nacc + 1);
                        mean = (1 - w) * prev + w * contribution;
                    } else {
                        err |= VPT_DEVERR_NONFINITE;
                    }
                    ++sample;
                    if (sample < P.spp) {
                        st = WS_CAMERA;
                    } else {
                        P.rng[pixel] = rng.state;
                        P.sum_rgb[3 * pixel] += sum_r;
                        P.sum_rgb[3 * pixel + 1] += sum_g;
                        P.sum_rgb[3 * pixel + 2] += sum_b;
                        P.mean_rgb[3 * pixel] = mean.r;
                        P.mean_rgb[3 * pixel + 1] = mean.g;
                        P.mean_rgb[3 * pixel + 2] = mean.b;
                        st = WS_FETCH;
                    }
                    break;
                }
                default:
                    st = WS_DONE;
                    break;
                }
            }
            if (st == WS_STEP) {
                push_track = true;
                W.seg0[slot] = make_float4(seg_eye.x, seg_eye.y, seg_eye.z, t);
                W.seg1[slot] = make_float4(seg_dir.x, seg_dir.y, seg_dir.z, t1);
                W.org[slot] = make_float4(origin.x, origin.y, origin.z, dir_pdf);
                W.dir[slot] = make_float4(dir.x, dir.y, dir.z, init_importance);
                W.tp[slot] = make_float4(throughput.r, throughput.g, throughput.b, area_pdf);
                W.contrib[slot] = make_float4(contribution.r, contribution.g, contribution.b, vis);
                W.emit[slot] = make_float4(emittance.r, emittance.g, emittance.b, 0.0f);
                W.rng[slot] = rng.state;
                W.pixel[slot] = pixel;
                W.sample[slot] = sample;
                W.path_length[slot] = path_length;
                W.rec[slot] = rec;
                W.flags[slot] = make_flags(WS_STEP, end_code, (flags & kFlagShadow) | (pick_sun ? kFlagPickSun : 0u));
                if (P.stream_mode != 1) {
                    W.sum[3 * slot] = sum_r;
                    W.sum[3 * slot + 1] = sum_g;
                    W.sum[3 * slot + 2] = sum_b;
                    W.mean[slot] = make_float4(mean.r, mean.g, mean.b, 0.0f);
                }
            }
        }
        warp_push(push_track, slot, W.track_queue + out_q * W.slots, W.count + out_q);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        n_vertices += __shfl_down_sync(0xffffffffu, n_vertices, o);
        n_samples += __shfl_down_sync(0xffffffffu, n_samples, o);
    }
    err = __reduce_or_sync(0xffffffffu, err);
    if ((threadIdx.x & 31) == 0) {
        if (n_vertices) atomicAdd(P.counters + 1, n_vertices);
        if (n_samples) atomicAdd(P.counters + 2, n_samples);
        if (err) atomicOr(P.error_flags, err);
    }
}

// ------------------------------------------------------------------------------ tracking kernel
template <bool kGridMajorant>
__global__ void __launch_bounds__(256) wf_track_kernel(const TraceParams P, const WfBuffers W, uint32_t in_q,
                                                       uint32_t pass_steps) {
    extern __shared__ float s_maj[];
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
    const uint32_t out_q = in_q ^ 1;
    const uint32_t n = W.count[in_q];
    const float global_maj = P.density_coeff * g.global_majorant;
    const uint32_t step_cap = P.max_steps > 0 ? static_cast<uint32_t>(P.max_steps) : kHardStepCap;
    const uint32_t lane = threadIdx.x & 31;

    int slot = -1;
    bool drained = false, shadow = false;
    V3 eye = v3(0, 0, 0), dir = v3(0, 0, 1);
    float t = 0, t1 = 0, vis = 1, maj = global_maj, texit = 0;
    uint32_t seg_steps = 0, pass_count = 0, rec_p = 0, rec_s = 0;
    Pcg32 rng{0};
    Dda dda;
    LeafCache leaf_cache;
    unsigned long long n_lookups = 0, n_cells = 0;
    unsigned int err = 0;

    while (true) {
        // Refill the lanes without a segment from the tracking queue (one atomic per warp).
        const bool want = slot < 0 && !drained;
        const uint32_t m = __ballot_sync(0xffffffffu, want);
        if (m) {
            const int leader = __ffs(m) - 1;
            uint32_t base = 0;
            if (static_cast<int>(lane) == leader) base = atomicAdd(W.count + 4, static_cast<uint32_t>(__popc(m)));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (want) {
                const uint32_t idx = base + __popc(m & ((1u << lane) - 1u));
                if (idx < n) {
                    slot = static_cast<int>(W.track_queue[in_q * W.slots + idx]);
                    const float4 s0 = W.seg0[slot], s1 = W.seg1[slot];
                    const uint32_t f = W.flags[slot];
                    eye = v3(s0.x, s0.y, s0.z);
                    t = s0.w;
                    dir = v3(s1.x, s1.y, s1.z);
                    t1 = s1.w;
                    shadow = f & kFlagShadow;
                    vis = W.contrib[slot].w;
                    rng.state = W.rng[slot];
                    const uint2 rc = W.rec[slot];
                    rec_p = rc.x;
                    rec_s = rc.y;
                    pass_count = 0;
                    if (f & kFlagResume) {
                        const int4 ds = W.dda_i[slot];
                        seg_steps = static_cast<uint32_t>(ds.w);
                        if constexpr (kGridMajorant) {
                            const float4 tn = W.dda_f[slot];
                            dda.cell[0] = ds.x;
                            dda.cell[1] = ds.y;
                            dda.cell[2] = ds.z;
                            dda.tnext[0] = tn.x;
                            dda.tnext[1] = tn.y;
                            dda.tnext[2] = tn.z;
                            dda_steps(g, dir, &dda);
                        }
                    } else {
                        seg_steps = 0;
                        if constexpr (kGridMajorant) dda_init(g, eye, dir, t, &dda);
                    }
                    if constexpr (kGridMajorant) {
                        texit = fminf(fminf(dda.tnext[0], dda.tnext[1]), fminf(dda.tnext[2], t1));
                        maj = P.density_coeff * cell_maj(maj_grid, g, dda);
                    } else {
                        maj = global_maj;
                    }
                } else {
                    drained = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, slot >= 0) == 0) break;

        // One step of every lane that holds a segment: advance to the next lookup (crossing
        // empty cells), look the density up, decide.
        uint32_t outcome = 0;  // 1 collision, 2 exit, 3 step cap, 4 suspended
        bool need_lookup = false;
        if (slot >= 0) {
            if constexpr (!kGridMajorant) {
                // optix_pathtracing_kernels.cu:113-118 / renderer_kernel_common.h:374-378.
                t += -logf(1.0f - rng.uniform()) / maj;
                if (!(t <= t1)) outcome = 2;  // also ends the segment on a NaN distance
                else need_lookup = true;
            } else {
                // Sample within the current cell; overshooting its exit restarts at the exit
                // (memoryless); empty cells are skipped without draws.
                while (true) {
                    if (maj > 0) {
                        float tt = t + -logf(1.0f - rng.uniform()) / maj;
                        if (tt < texit) {
                            t = tt;
                            need_lookup = true;
                            break;
                        }
                    }
                    t = texit;
                    if (texit >= t1) {
                        outcome = 2;
                        break;
                    }
                    bool ax0 = dda.tnext[0] <= dda.tnext[1] && dda.tnext[0] <= dda.tnext[2];
                    bool ax1 = !ax0 && dda.tnext[1] <= dda.tnext[2];
                    bool ax2 = !ax0 && !ax1;
                    if (ax0) dda.cell[0] += dda.step[0];
                    if (ax1) dda.cell[1] += dda.step[1];
                    if (ax2) dda.cell[2] += dda.step[2];
                    ++n_cells;
                    if (dda.cell[0] < 0 || dda.cell[0] >= g.mx || dda.cell[1] < 0 || dda.cell[1] >= g.my ||
                        dda.cell[2] < 0 || dda.cell[2] >= g.mz) {
                        t = t1;
                        outcome = 2;
                        break;
                    }
                    if (ax0) dda.tnext[0] += dda.tdelta[0];
                    if (ax1) dda.tnext[1] += dda.tdelta[1];
                    if (ax2) dda.tnext[2] += dda.tdelta[2];
                    texit = fminf(fminf(dda.tnext[0], dda.tnext[1]), fminf(dda.tnext[2], t1));
                    maj = P.density_coeff * cell_maj(maj_grid, g, dda);
                }
            }
        }
        if (need_lookup) {
            const V3 pos = eye + dir * t;
            const float density = P.density_coeff * sample_trilinear(g, world_to_index(g, pos), leaf_cache);
            ++n_lookups;
            ++seg_steps;
            ++pass_count;
            if (shadow) {
                ++rec_s;
                vis *= (1 - density / maj);
                if (vis < P.shadow_rr) {
                    const float q = vis / P.shadow_rr;
                    if (rng.uniform() >= q) {
                        vis = 0.0f;
                        outcome = 2;
                    } else {
                        vis = P.shadow_rr;
                    }
                }
            } else {
                ++rec_p;
                if (rng.uniform() < density / maj) outcome = 1;
            }
            if (outcome == 0 && seg_steps >= step_cap) {
                err |= VPT_DEVERR_STEP_CAP;
                outcome = 3;
            }
            if (outcome == 0 && pass_count >= pass_steps) outcome = 4;
        }
        bool to_event = false, to_track = false;
        if (outcome != 0) {
            W.rng[slot] = rng.state;
            W.rec[slot] = make_uint2(rec_p, rec_s);
            const uint32_t f = W.flags[slot] & (kFlagShadow | kFlagPickSun | 0xFF00u);
            if (outcome == 4) {
                W.seg0[slot] = make_float4(eye.x, eye.y, eye.z, t);
                W.contrib[slot].w = vis;
                W.dda_i[slot] = make_int4(dda.cell[0], dda.cell[1], dda.cell[2], static_cast<int>(seg_steps));
                if constexpr (kGridMajorant) W.dda_f[slot] = make_float4(dda.tnext[0], dda.tnext[1], dda.tnext[2], 0.0f);
                W.flags[slot] = (f & ~0xFFu) | WS_STEP | kFlagResume;
                to_track = true;
            } else {
                uint32_t st;
                uint32_t fl = f & ~(0xFFu | kFlagResume);
                if (outcome == 1) {
                    st = WS_VERTEX;
                    W.seg0[slot].w = t;
                } else if (outcome == 2) {
                    st = shadow ? WS_NEE_DONE : WS_ESCAPE;
                    if (shadow) W.contrib[slot].w = vis;
                } else {
                    st = WS_END_SAMPLE;
                    fl = (fl & ~0xFF00u) | (WE_STEP_CAP << 8);
                }
                W.flags[slot] = fl | st;
                to_event = true;
            }
        }
        warp_push(to_event, static_cast<uint32_t>(slot), W.event_queue + out_q * W.slots, W.count + 2 + out_q);
        warp_push(to_track, static_cast<uint32_t>(slot), W.track_queue + out_q * W.slots, W.count + out_q);
        if (outcome != 0) slot = -1;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        n_lookups += __shfl_down_sync(0xffffffffu, n_lookups, o);
        n_cells += __shfl_down_sync(0xffffffffu, n_cells, o);
    }
    err = __reduce_or_sync(0xffffffffu, err);
    if ((threadIdx.x & 31) == 0) {
        if (n_lookups) atomicAdd(P.counters + 0, n_lookups);
        if (n_cells) atomicAdd(P.counters + 3, n_cells);
        if (err) atomicOr(P.error_flags, err);
    }
}

}  // namespace

const void* wf_track_kernel_ptr(bool grid_majorant) {
    return grid_majorant ? reinterpret_cast<const void*>(wf_track_kernel<true>)
                         : reinterpret_cast<const void*>(wf_track_kernel<false>);
}

void VptContextImpl::release_wf() {
    WfBuffers& W = wf;
    void* ptrs[] = {W.rng, W.pixel, W.sample, W.path_length, W.flags, W.rec, W.org, W.dir, W.tp, W.contrib,
                    W.emit, W.seg0, W.seg1, W.dda_i, W.dda_f, W.sum, W.mean, W.track_queue, W.event_queue, W.count};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    W = WfBuffers{};
    if (wf_pinned) cudaFreeHost(wf_pinned);
    wf_pinned = nullptr;
    for (cudaEvent_t& e : wf_events) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
    }
}

namespace {
template <typename T>
bool wf_alloc(T** p, size_t count) {
    return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T)) == cudaSuccess;
}
}  // namespace

int wf_ensure(VptContextImpl* c, uint32_t slots) {
    if (c->wf.capacity >= slots && c->wf.count) {
        c->wf.slots = slots;
        return VPT_OK;
    }
    c->release_wf();
    WfBuffers& W = c->wf;
    const size_t n = slots;
    const bool ok = wf_alloc(&W.rng, n) && wf_alloc(&W.pixel, n) && wf_alloc(&W.sample, n) &&
                    wf_alloc(&W.path_length, n) && wf_alloc(&W.flags, n) && wf_alloc(&W.rec, n) && wf_alloc(&W.org, n) &&
                    wf_alloc(&W.dir, n) && wf_alloc(&W.tp, n) && wf_alloc(&W.contrib, n) && wf_alloc(&W.emit, n) &&
                    wf_alloc(&W.seg0, n) && wf_alloc(&W.seg1, n) && wf_alloc(&W.dda_i, n) && wf_alloc(&W.dda_f, n) &&
                    wf_alloc(&W.sum, 3 * n) && wf_alloc(&W.mean, n) && wf_alloc(&W.track_queue, 2 * n) &&
                    wf_alloc(&W.event_queue, 2 * n) && wf_alloc(&W.count, 8);
    if (!ok) {
        c->release_wf();
        return ctx_set_error(VPT_ERR_OUT_OF_MEMORY, "wavefront: cudaMalloc of the path state failed");
    }
    W.slots = slots;
    W.capacity = slots;
    return VPT_OK;
}

int wf_run(VptContextImpl* c, const TraceParams& tp, bool grid_majorant, size_t smem, cudaStream_t s) {
    WfBuffers& W = c->wf;
    int per_sm = c->wf_track_ctas_per_sm;
    if (per_sm <= 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wf_track_kernel_ptr(grid_majorant), 256,
                                                          grid_majorant ? smem : 0) != cudaSuccess ||
            per_sm <= 0)
            per_sm = 1;
    }
    const int track_ctas = c->num_sms * per_sm;
    const int event_ctas = c->num_sms * 8;
    const uint32_t pass_steps = c->wf_pass_steps > 0 ? static_cast<uint32_t>(c->wf_pass_steps) : 64u;
    // pinned ring of tracking-queue counts read back with a lag of kLag passes
    constexpr int kRing = 8, kLag = 3;
    if (!c->wf_pinned) {
        if (cudaMallocHost(reinterpret_cast<void**>(&c->wf_pinned), kRing * sizeof(uint32_t)) != cudaSuccess)
            return ctx_set_error(VPT_ERR_OUT_OF_MEMORY, "wavefront: pinned counters");
        for (int i = 0; i < kRing; ++i) {
            if (cudaEventCreateWithFlags(&c->wf_events[i], cudaEventDisableTiming) != cudaSuccess)
                return ctx_set_error(VPT_ERR_CUDA, "wavefront: events");
        }
    }
    cudaMemsetAsync(W.count, 0, 8 * sizeof(uint32_t), s);
    const uint32_t max_passes = 1u << 22;
    for (uint32_t pass = 0; pass < max_passes; ++pass) {
        const uint32_t q = pass & 1u;
        wf_event_kernel<<<event_ctas, 128, 0, s>>>(tp, W, pass == 0 ? 1 : 0, q, q);
        cudaMemcpyAsync(c->wf_pinned + pass % kRing, W.count + q, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        cudaEventRecord(c->wf_events[pass % kRing], s);
        if (grid_majorant)
            wf_track_kernel<true><<<track_ctas, 256, smem, s>>>(tp, W, q, pass_steps);
        else
            wf_track_kernel<false><<<track_ctas, 256, 0, s>>>(tp, W, q, pass_steps);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return ctx_set_error(VPT_ERR_CUDA, cudaGetErrorString(e));
        if (pass >= static_cast<uint32_t>(kLag)) {
            const uint32_t check = pass - kLag;
            if (cudaEventSynchronize(c->wf_events[check % kRing]) != cudaSuccess)
                return ctx_set_error(VPT_ERR_CUDA, "wavefront: event synchronize");
            if (c->wf_pinned[check % kRing] == 0) return VPT_OK;  // every slot retired at that pass
        }
    }
    return ctx_set_error(VPT_ERR_CUDA, "wavefront: pass limit reached");
}

}  // namespace vpt

extern "C" int vpt_set_tracker(VptContext* c, int32_t kind, int32_t slots_per_sm, int32_t pass_steps,
                               int32_t track_ctas_per_sm) {
    if (!c || kind < 0 || kind > 1 || slots_per_sm < 0 || pass_steps < 0 || track_ctas_per_sm < 0)
        return vpt::ctx_set_error(VPT_ERR_INVALID_ARGUMENT, "vpt_set_tracker: bad arguments");
    c->tracker = kind;
    c->wf_slots_per_sm = slots_per_sm;
    c->wf_pass_steps = pass_steps;
    c->wf_track_ctas_per_sm = track_ctas_per_sm;
    return VPT_OK;
}
