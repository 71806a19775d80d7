// Device-side building blocks of the volumetric path tracer: RNG, vector math, frames,
// phase functions, the sparse density grid, environment sampling and the majorant DDA.
// Citations are file:line within the reference project (shocker-0x15/rtcamp8).
//
// Every routine that decides a path event is written so that its float operations happen
// in the same order as the reference code; the tracker translation unit is compiled
// without fused multiply-add contraction so those decisions reproduce the reference
// estimator's random-number-by-random-number behaviour.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vpt {

constexpr float kPi = 3.14159265358979323846f;

// ------------------------------------------------------------------------------ vectors
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// basic_types.h:850-853: v /= length() multiplies by the reciprocal.
__device__ __forceinline__ V3 normalize(V3 a) {
    float r = 1.0f / sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    return a * r;
}

struct RGB {
    float r, g, b;
};
__device__ __forceinline__ RGB rgb(float r, float g, float b) { return RGB{r, g, b}; }
__device__ __forceinline__ RGB operator+(RGB a, RGB b) { return rgb(a.r + b.r, a.g + b.g, a.b + b.b); }
__device__ __forceinline__ RGB operator*(RGB a, RGB b) { return rgb(a.r * b.r, a.g * b.g, a.b * b.b); }
__device__ __forceinline__ RGB operator*(RGB a, float s) { return rgb(a.r * s, a.g * s, a.b * s); }
__device__ __forceinline__ RGB operator*(float s, RGB a) { return rgb(s * a.r, s * a.g, s * a.b); }
__device__ __forceinline__ RGB rdiv(RGB a, float s) {
    float r = 1.0f / s;
    return a * r;
}
// basic_types.h:2981-2986.
__device__ __forceinline__ float luminance(RGB c) {
    return 0.2126729f * c.r + 0.7151522f * c.g + 0.0721750f * c.b;
}
__device__ __forceinline__ bool all_nonneg_finite(RGB c) {
    return isfinite(c.r) && isfinite(c.g) && isfinite(c.b) && c.r >= 0.0f && c.g >= 0.0f && c.b >= 0.0f;
}

// ------------------------------------------------------------------------------ PCG32
// common_renderer_types.h:101-125: 64-bit LCG, XSH-RR output, [0,1) float from 23 bits.
struct Pcg32 {
    uint64_t state;
    __device__ __forceinline__ uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + 1ULL;
        uint32_t xorshifted = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = static_cast<uint32_t>(old >> 59u);
        return __funnelshift_r(xorshifted, xorshifted, rot);
    }
    __device__ __forceinline__ float uniform() {
        return __uint_as_float((next() >> 9) | 0x3f800000u) - 1.0f;
    }
};

// Jump-ahead of a PCG32 state by `delta` draws (O(log delta) LCG advance, Brown 1994).
__device__ __forceinline__ uint64_t pcg_advance(uint64_t state, uint64_t delta) {
    uint64_t cur_mult = 6364136223846793005ULL, cur_plus = 1ULL;
    uint64_t acc_mult = 1ULL, acc_plus = 0ULL;
    while (delta > 0) {
        if (delta & 1ULL) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1ULL) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1;
    }
    return acc_mult * state + acc_plus;
}
// Sample-parallel streams: sample s of a pixel starts 2^40 * s draws into the pixel's stream.
constexpr int kSampleStreamShift = 40;

// ------------------------------------------------------------------------------ frames
// common_renderer_types.h:1379-1405 with basic_types.h:857-864.
struct Frame {
    V3 t, b, n;
};
__device__ __forceinline__ Frame make_frame(V3 n) {
    float sign = n.z >= 0 ? 1.0f : -1.0f;
    float a = -1 / (sign + n.z);
    float b = n.x * n.y * a;
    Frame f;
    f.t = v3(1 + sign * n.x * n.x * a, sign * b, -sign * n.x);
    f.b = v3(b, sign + n.y * n.y * a, -n.y);
    f.n = n;
    return f;
}
__device__ __forceinline__ V3 to_local(const Frame& f, V3 v) { return v3(dot(f.t, v), dot(f.b, v), dot(f.n, v)); }
__device__ __forceinline__ V3 from_local(const Frame& f, V3 v) {
    return v3(dot(v3(f.t.x, f.b.x, f.n.x), v), dot(v3(f.t.y, f.b.y, f.n.y), v), dot(v3(f.t.z, f.b.z, f.n.z), v));
}

// basic_types.h:870-874 / 900-907.
__device__ __forceinline__ void to_polar_yup(V3 v, float* theta, float* phi) {
    *theta = acosf(fminf(fmaxf(v.y, -1.0f), 1.0f));
    *phi = fmodf(atan2f(-v.x, v.z) + 2 * kPi, 2 * kPi);
}
// The same result without the library remainder: for a = atan2(..) in [-pi, pi] the sum lies in
// [pi, 3 pi], where fmod is one subtraction of 2 pi, exact by Sterbenz's lemma, so both forms agree
// bit for bit. The radiance-cache passes use this one (their render samples mostly end at an
// environment hit and write cache queries: render pass 4.76 -> 4.53 ms per 128 spp at 256^2);
// the plain tracer keeps the library call, because the select changes its register allocation at
// its 72-register bound (spills; C2 35.0 -> 37.8 ms).
__device__ __forceinline__ void to_polar_yup_sel(V3 v, float* theta, float* phi) {
    *theta = acosf(fminf(fmaxf(v.y, -1.0f), 1.0f));
    const float a = atan2f(-v.x, v.z) + 2 * kPi;
    *phi = a >= 2 * kPi ? a - 2 * kPi : a;
}
__device__ __forceinline__ V3 from_polar_yup(float phi, float theta) {
    float sp = sinf(phi), cp = cosf(phi);
    float st = sinf(theta), ct = cosf(theta);
    return v3(-sp * st, ct, cp * st);
}

// basic_types.h:1620-1628 (columns) and :2131-2134 (M * v as row dot products).
struct M3 {
    V3 c0, c1, c2;
};
__device__ __forceinline__ M3 quat_to_m3(float x, float y, float z, float w) {
    float xx = x * x, yy = y * y, zz = z * z;
    float xy = x * y, yz = y * z, zx = z * x;
    float xw = x * w, yw = y * w, zw = z * w;
    M3 m;
    m.c0 = v3(1 - 2 * (yy + zz), 2 * (xy + zw), 2 * (zx - yw));
    m.c1 = v3(2 * (xy - zw), 1 - 2 * (xx + zz), 2 * (yz + xw));
    m.c2 = v3(2 * (zx + yw), 2 * (yz - xw), 1 - 2 * (xx + yy));
    return m;
}
__device__ __forceinline__ V3 mul(const M3& m, V3 v) {
    return v3(dot(v3(m.c0.x, m.c1.x, m.c2.x), v), dot(v3(m.c0.y, m.c1.y, m.c2.y), v),
              dot(v3(m.c0.z, m.c1.z, m.c2.z), v));
}

// ------------------------------------------------------------------------------ grid
// Sparse density grid: NanoVDB-style 8^3 leaves (value order x<<6 | y<<3 | z) reached
// through a dense table over leaf cells. Voxels outside the index box or in absent
// leaves read the background value 0.
struct Grid {
    const int32_t* __restrict__ leaf_table;   // lx*ly*lz, slot or -1
    const float* __restrict__ leaf_values;    // slot * 512 + local
    const float* __restrict__ cell_majorant;  // lx*ly*lz (8^3-voxel cells)
    // Majorant grid of the DDA: cells of 2^maj_shift voxels (maj_shift >= 3), max-pooled from
    // the 8^3-voxel cells, mx*my*mz values.
    const float* __restrict__ maj;
    int32_t mx, my, mz, maj_shift;
    int32_t nx, ny, nz;
    int32_t lx, ly, lz;
    float inv_voxel_size;
    float origin[3];
    float bbox_min[3], bbox_max[3];
    float global_majorant;
};

__device__ __forceinline__ int32_t leaf_slot(const Grid& g, int cx, int cy, int cz) {
    return __ldg(g.leaf_table + (static_cast<int64_t>(cx) * g.ly + cy) * g.lz + cz);
}
__device__ __forceinline__ float grid_value(const Grid& g, int x, int y, int z) {
    if (static_cast<uint32_t>(x) >= static_cast<uint32_t>(g.nx) || static_cast<uint32_t>(y) >= static_cast<uint32_t>(g.ny) ||
        static_cast<uint32_t>(z) >= static_cast<uint32_t>(g.nz))
        return 0.0f;
    int32_t slot = leaf_slot(g, x >> 3, y >> 3, z >> 3);
    if (slot < 0) return 0.0f;
    return __ldg(g.leaf_values + static_cast<int64_t>(slot) * 512 + (((x & 7) << 6) | ((y & 7) << 3) | (z & 7)));
}

// NanoVDB.h:1409-1414 / 2029-2032 (inverse map of a scale + translate transform).
__device__ __forceinline__ V3 world_to_index(const Grid& g, V3 p) {
    return v3((p.x - g.origin[0]) * g.inv_voxel_size, (p.y - g.origin[1]) * g.inv_voxel_size,
              (p.z - g.origin[2]) * g.inv_voxel_size);
}

// The last leaf a lane looked up: successive tracking steps along a ray mostly stay in the
// same 8^3 leaf, so the table read (a dependent load before the voxel loads) is skipped.
struct LeafCache {
    int32_t key = -1;
    int32_t slot = -1;
};

// util/SampleFromVoxels.h:419-459: first-order sampler, lerps along z, then y, then x.
// When the 2x2x2 stencil lies inside one leaf (about 2/3 of the lookups) it reads one
// table entry (or the lane's cached one) and eight values of that leaf.
struct Stencil {
    float wx, wy, wz;
    int i, j, k;
    bool fast;    // inside the grid and inside one leaf
    int32_t key;  // that leaf's table index
};

__device__ __forceinline__ Stencil stencil_at(const Grid& g, V3 xyz) {
    Stencil s;
    const float fi = floorf(xyz.x), fj = floorf(xyz.y), fk = floorf(xyz.z);
    s.wx = xyz.x - fi;
    s.wy = xyz.y - fj;
    s.wz = xyz.z - fk;
    s.i = static_cast<int>(fi);
    s.j = static_cast<int>(fj);
    s.k = static_cast<int>(fk);
    const bool inside = static_cast<uint32_t>(s.i) < static_cast<uint32_t>(g.nx - 1) &&
                        static_cast<uint32_t>(s.j) < static_cast<uint32_t>(g.ny - 1) &&
                        static_cast<uint32_t>(s.k) < static_cast<uint32_t>(g.nz - 1);
    s.fast = inside && (s.i & 7) != 7 && (s.j & 7) != 7 && (s.k & 7) != 7;
    s.key = ((s.i >> 3) * g.ly + (s.j >> 3)) * g.lz + (s.k >> 3);
    return s;
}

// Table entry of a fast stencil's leaf through the lane's one-entry cache.
__device__ __forceinline__ int32_t stencil_slot(const Grid& g, const Stencil& s, LeafCache& cache) {
    if (s.key == cache.key) return cache.slot;
    const int32_t slot = __ldg(g.leaf_table + s.key);
    cache.key = s.key;
    cache.slot = slot;
    return slot;
}

// v = v000, v001, v010, v011, v100, v101, v110, v111 (x, y, z bits).
__device__ __forceinline__ void stencil_load_fast(const Grid& g, const Stencil& s, int32_t slot, float (&v)[8]) {
    const float* p = g.leaf_values + static_cast<int64_t>(slot) * 512 + (((s.i & 7) << 6) | ((s.j & 7) << 3) | (s.k & 7));
    v[0] = __ldg(p);
    v[1] = __ldg(p + 1);
    v[2] = __ldg(p + 8);
    v[3] = __ldg(p + 9);
    v[4] = __ldg(p + 64);
    v[5] = __ldg(p + 65);
    v[6] = __ldg(p + 72);
    v[7] = __ldg(p + 73);
}

__device__ __forceinline__ void stencil_load_slow(const Grid& g, const Stencil& s, float (&v)[8]) {
    v[0] = grid_value(g, s.i, s.j, s.k);
    v[1] = grid_value(g, s.i, s.j, s.k + 1);
    v[2] = grid_value(g, s.i, s.j + 1, s.k);
    v[3] = grid_value(g, s.i, s.j + 1, s.k + 1);
    v[4] = grid_value(g, s.i + 1, s.j, s.k);
    v[5] = grid_value(g, s.i + 1, s.j, s.k + 1);
    v[6] = grid_value(g, s.i + 1, s.j + 1, s.k);
    v[7] = grid_value(g, s.i + 1, s.j + 1, s.k + 1);
}

__device__ __forceinline__ float stencil_lerp(const Stencil& s, const float (&v)[8]) {
    auto lerp = [](float a, float b, float w) { return a + w * (b - a); };
    float vy = lerp(v[0], v[1], s.wz);
    float vy1 = lerp(v[2], v[3], s.wz);
    const float vx = lerp(vy, vy1, s.wy);
    vy1 = lerp(v[6], v[7], s.wz);
    vy = lerp(v[4], v[5], s.wz);
    const float vx1 = lerp(vy, vy1, s.wy);
    return lerp(vx, vx1, s.wx);
}

__device__ __forceinline__ float sample_trilinear(const Grid& g, V3 xyz, LeafCache& cache) {
    const Stencil s = stencil_at(g, xyz);
    float v[8];
    if (s.fast) {
        const int32_t slot = stencil_slot(g, s, cache);
        if (slot < 0) return 0.0f;
        stencil_load_fast(g, s, slot, v);
    } else {
        stencil_load_slow(g, s, v);
    }
    return stencil_lerp(s, v);
}

// ------------------------------------------------------------------------------ leaf staging
// Per-warp copy of one 8^3 leaf (2 KB) in shared memory. When at least `min_lanes` lanes of a
// warp look up inside the same leaf in one tracking step, the leaf is brought in with one bulk
// asynchronous copy (cp.async.bulk, global -> shared, completion counted in bytes on the warp's
// mbarrier), and the lanes of that leaf read their eight stencil values from shared memory
// (the same bits as from global memory, so the decisions do not change).
constexpr uint32_t kLeafBytes = 512 * sizeof(float);
constexpr uint32_t kStageWaitLimit = 1u << 22;

struct LeafStage {
    float* values;    // this warp's buffer (16-byte aligned)
    uint64_t* bar;    // this warp's mbarrier
    int32_t key;      // staged leaf's table index; -1 = none, -2 = staging switched off (timeout)
    int32_t slot;     // its slot (-1: an empty leaf, every value 0)
    uint32_t phase;   // parity of the next completion of `bar`
};

__device__ __forceinline__ uint32_t smem_addr32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void stage_bar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Issued by one lane: the previous contents were read by the generic proxy, hence the proxy fence.
__device__ __forceinline__ void stage_copy(float* dst, const float* src, uint64_t* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(smem_addr32(bar)), "r"(kLeafBytes)
                 : "memory");
    (void)state;
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr32(dst)),
                 "l"(src), "r"(kLeafBytes), "r"(smem_addr32(bar))
                 : "memory");
}
// Bounded wait for the copy's completion (false after kStageWaitLimit polls).
__device__ __forceinline__ bool stage_wait(uint64_t* bar, uint32_t phase) {
    for (uint32_t i = 0; i < kStageWaitLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(smem_addr32(bar)), "r"(phase)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// sample_trilinear with the warp's staged leaf. Called by all 32 lanes together; `need` says
// whether this lane wants a value at `xyz`. Sets `timed_out` if a copy did not complete (the
// warp then stops staging; see the tracker's exit).
__device__ __forceinline__ float sample_trilinear_staged(const Grid& g, bool need, V3 xyz, LeafCache& cache,
                                                         LeafStage& st, int min_lanes, bool& timed_out) {
    const uint32_t lane = threadIdx.x & 31;
    const Stencil s = stencil_at(g, xyz);
    const bool cand = need && s.fast;
    const int key = cand ? s.key : -1 - static_cast<int>(lane);  // non-candidates in groups of one
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    const uint32_t score = cand ? (static_cast<uint32_t>(__popc(peers)) << 5) | lane : 0u;
    const uint32_t best = __reduce_max_sync(0xffffffffu, score);
    if (st.key != -2 && static_cast<int>(best >> 5) >= min_lanes) {
        const int best_lane = static_cast<int>(best & 31);
        const int leaf = __shfl_sync(0xffffffffu, key, best_lane);
        if (leaf != st.key) {
            int32_t slot = 0;
            if (static_cast<int>(lane) == best_lane) slot = stencil_slot(g, s, cache);
            slot = __shfl_sync(0xffffffffu, slot, best_lane);
            if (slot >= 0) {
                __syncwarp();  // every lane's reads of the previous leaf are complete
                if (lane == 0) stage_copy(st.values, g.leaf_values + static_cast<int64_t>(slot) * 512, st.bar);
                const bool ok = __all_sync(0xffffffffu, stage_wait(st.bar, st.phase));
                st.phase ^= 1u;
                if (ok) {
                    st.key = leaf;
                    st.slot = slot;
                } else {
                    st.key = -2;
                    timed_out = true;
                }
            } else {
                st.key = leaf;
                st.slot = -1;
            }
        }
    }
    if (!need) return 0.0f;
    float v[8];
    if (s.fast && s.key == st.key) {
        if (st.slot < 0) return 0.0f;
        const float* p = st.values + (((s.i & 7) << 6) | ((s.j & 7) << 3) | (s.k & 7));
        v[0] = p[0];
        v[1] = p[1];
        v[2] = p[8];
        v[3] = p[9];
        v[4] = p[64];
        v[5] = p[65];
        v[6] = p[72];
        v[7] = p[73];
    } else if (s.fast) {
        const int32_t slot = stencil_slot(g, s, cache);
        if (slot < 0) return 0.0f;
        stencil_load_fast(g, s, slot, v);
    } else {
        stencil_load_slow(g, s, v);
    }
    return stencil_lerp(s, v);
}

// util/Ray.h:343-363 + :512-520 (slab test, clipped to the ray's [tmin, tmax]).
__device__ __forceinline__ bool clip_ray(V3 bmin, V3 bmax, V3 eye, V3 dir, float tmin, float tmax, float* t0o,
                                         float* t1o) {
    float ix = 1 / dir.x, iy = 1 / dir.y, iz = 1 / dir.z;
    bool sx = ix < 0, sy = iy < 0, sz = iz < 0;
    float t0 = ((sx ? bmax.x : bmin.x) - eye.x) * ix;
    float t2 = ((sy ? bmin.y : bmax.y) - eye.y) * iy;
    if (t0 > t2) return false;
    float t1 = ((sx ? bmin.x : bmax.x) - eye.x) * ix;
    float t3 = ((sy ? bmax.y : bmin.y) - eye.y) * iy;
    if (t3 > t1) return false;
    if (t3 > t0) t0 = t3;
    if (t2 < t1) t1 = t2;
    t3 = ((sz ? bmax.z : bmin.z) - eye.z) * iz;
    if (t3 > t1) return false;
    t2 = ((sz ? bmin.z : bmax.z) - eye.z) * iz;
    if (t0 > t2) return false;
    if (t3 > t0) t0 = t3;
    if (tmax < t0) return false;
    if (t2 < t1) t1 = t2;
    if (tmin > t1) return false;
    if (tmin > t0) t0 = tmin;
    if (tmax < t1) t1 = tmax;
    *t0o = t0;
    *t1o = t1;
    return true;
}

// ------------------------------------------------------------------------------ phase
// common_renderer_types.h:2063-2097 (Schlick, local z = -cos(theta)); Henyey-Greenstein in
// the same convention.
__device__ __forceinline__ float phase_value(int kind, float g, float cos_theta) {
    if (kind == 0) {
        float d = 1 - g * cos_theta;
        return (1 - g * g) / (4 * kPi * (d * d));
    }
    float d = 1 + g * g - 2 * g * cos_theta;
    return (1 - g * g) / (4 * kPi * (d * sqrtf(d)));
}
__device__ __forceinline__ float phase_pdf(int kind, float g, V3 local) { return phase_value(kind, g, -local.z); }
__device__ __forceinline__ float phase_sample(int kind, float g, float u0, float u1, V3* local) {
    float cos_theta;
    if (kind == 0) {
        cos_theta = (2 * u1 + g - 1) / (2 * g * u1 - g + 1);
    } else if (fabsf(g) < 1e-3f) {
        cos_theta = 1 - 2 * u1;
    } else {
        float sq = (1 - g * g) / (1 - g + 2 * g * u1);
        cos_theta = (1 + g * g - sq * sq) / (2 * g);
    }
    cos_theta = fminf(fmaxf(cos_theta, -1.0f), 1.0f);
    float phi = 2 * kPi * u0;
    float value = phase_value(kind, g, cos_theta);
    float sin_theta = sqrtf(1 - cos_theta * cos_theta);
    *local = v3(cosf(phi) * sin_theta, sinf(phi) * sin_theta, -cos_theta);
    return value;
}

// ------------------------------------------------------------------------------ environment
struct Env {
    const float4* __restrict__ texels;   // w*h RGB(A), point sampled
    const float* __restrict__ mips;      // importance mip chain
    int64_t mip_offset[16];
    int32_t w, h;
    int32_t map_w, map_h, num_mips;
    float integral;
    float power, rotation;
};

__device__ __forceinline__ int env_x(const Env& e, float u) { return min(max(static_cast<int>(u * e.w), 0), e.w - 1); }
__device__ __forceinline__ int env_y(const Env& e, float v) { return min(max(static_cast<int>(v * e.h), 0), e.h - 1); }
__device__ __forceinline__ RGB env_texel(const Env& e, int x, int y) {
    float4 t = __ldg(e.texels + static_cast<int64_t>(y) * e.w + x);
    return rgb(t.x, t.y, t.z);
}
__device__ __forceinline__ float mip_texel(const Env& e, int level, int x, int y) {
    int w = max(e.map_w >> level, 1);
    return __ldg(e.mips + e.mip_offset[level] + static_cast<int64_t>(y) * w + x);
}

// common_renderer_types.h:479-548.
__device__ __forceinline__ void imp_sample(const Env& e, float u0, float u1, int* px, int* py, float* ru0,
                                           float* ru1, float* prob) {
    int ix = 0, iy = 0;
    float p = 1;
    int cur_w = 2, cur_h = e.map_w > e.map_h ? 1 : 2;
    for (int level = e.num_mips - 2; level >= 0; --level) {
        ix *= 2;
        iy *= 2;
        bool has_lower = (iy + 1.5f) < cur_h;
        bool has_right = (ix + 1.5f) < cur_w;
        float vul = mip_texel(e, level, ix, iy);
        float vur = has_right ? mip_texel(e, level, ix + 1, iy) : 0.0f;
        float vll = has_lower ? mip_texel(e, level, ix, iy + 1) : 0.0f;
        float vlr = (has_right && has_lower) ? mip_texel(e, level, ix + 1, iy + 1) : 0.0f;
        float left = vll + vul;
        float right = vlr + vur;
        u0 *= (left + right);
        p *= 1.0f / (left + right);
        float upper, lower;
        if (u0 < left) {
            u0 = (u0 - 0) / left;
            upper = vul;
            lower = vll;
        } else {
            ix += 1;
            u0 = (u0 - left) / right;
            upper = vur;
            lower = vlr;
        }
        u1 *= (upper + lower);
        if (u1 < upper) {
            p *= upper;
            u1 = (u1 - 0) / upper;
        } else {
            iy += 1;
            p *= lower;
            u1 = (u1 - upper) / lower;
        }
        // Only an all-zero map can step outside the level (0 / 0 picks the right column).
        ix = min(ix, cur_w - 1);
        iy = min(iy, cur_h - 1);
        cur_w *= 2;
        cur_h *= 2;
    }
    *px = ix;
    *py = iy;
    *ru0 = u0;
    *ru1 = u1;
    *prob = p;
}

// common_renderer_types.h:2419-2440 + :987-1000.
__device__ __forceinline__ RGB env_sample(const Env& e, float u0, float u1, V3* dir, float* dir_pdf) {
    float prob;
    int px, py;
    imp_sample(e, u0, u1, &px, &py, &u0, &u1, &prob);
    float u = (px + u0) / e.w;
    float v = (py + u1) / e.h;
    float uv_pdf = static_cast<float>(static_cast<uint32_t>(e.w) * static_cast<uint32_t>(e.h)) * prob;
    float phi = 2 * kPi * u;
    float theta = kPi * v;
    float pdf = uv_pdf / (2 * (kPi * kPi) * sinf(theta));
    RGB radiance;
    if (!isfinite(pdf)) {
        pdf = 0.0f;
        radiance = rgb(0, 0, 0);
    } else {
        radiance = env_texel(e, env_x(e, u), env_y(e, v));
    }
    *dir_pdf = pdf;
    radiance = e.power * radiance;
    float pos_phi = phi - e.rotation;
    pos_phi = pos_phi - floorf(pos_phi / (2 * kPi)) * 2 * kPi;
    *dir = from_polar_yup(pos_phi, theta);
    return radiance;
}

// common_renderer_types.h:2442-2458 + :1002-1013.
template <bool kSelPolar = false>
__device__ __forceinline__ RGB env_evaluate(const Env& e, V3 dir, float* hyp_pdf) {
    float theta, pos_phi;
    if constexpr (kSelPolar)
        to_polar_yup_sel(dir, &theta, &pos_phi);
    else
        to_polar_yup(dir, &theta, &pos_phi);
    float phi = pos_phi + e.rotation;
    phi = phi - floorf(phi / (2 * kPi)) * 2 * kPi;
    float u = phi / (2 * kPi), v = theta / kPi;
    int tx = env_x(e, u), ty = env_y(e, v);
    RGB radiance = env_texel(e, tx, ty);
    float prob = mip_texel(e, 0, tx, ty) / e.integral;
    float uv_pdf = static_cast<float>(static_cast<uint32_t>(e.w) * static_cast<uint32_t>(e.h)) * prob;
    float pdf = uv_pdf / (2 * (kPi * kPi) * sinf(theta));
    if (!isfinite(pdf)) {
        pdf = 0.0f;
        radiance = rgb(0, 0, 0);
    }
    *hyp_pdf = pdf;
    return e.power * radiance;
}

}  // namespace vpt
