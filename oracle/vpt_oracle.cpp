/*
 * ORACLE (test infrastructure only) — CPU restatement of the reference's plain volumetric
 * path tracer. See vpt_oracle.h for the parity status. Citations are file:line within the
 * reference project (shocker-0x15/rtcamp8).
 *
 * Built with -ffp-contract=off so x86-64 and aarch64 hosts produce identical bits.
 * Random-draw order where the reference leaves it unspecified (two rng draws as arguments
 * of one call: optix_pathtracing_kernels.cu:341, renderer_kernel_common.h:321-324) is pinned
 * left to right: the first draw feeds the first parameter.
 */
#include "vpt_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr float kPi = 3.14159265358979323846f;

struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
// basic_types.h:850-853 and :817-820: v /= length() is a multiply by 1 / length.
inline V3 normalize(V3 a) {
    float r = 1.0f / length(a);
    return a * r;
}

struct RGB {
    float r, g, b;
};
inline RGB rgb(float r, float g, float b) { return RGB{r, g, b}; }
inline RGB operator+(RGB a, RGB b) { return rgb(a.r + b.r, a.g + b.g, a.b + b.b); }
inline RGB operator*(RGB a, RGB b) { return rgb(a.r * b.r, a.g * b.g, a.b * b.b); }
inline RGB operator*(RGB a, float s) { return rgb(a.r * s, a.g * s, a.b * s); }
inline RGB operator*(float s, RGB a) { return rgb(s * a.r, s * a.g, s * a.b); }
// basic_types.h:2939-2942: RGB / s multiplies by 1 / s.
inline RGB div(RGB a, float s) {
    float r = 1.0f / s;
    return a * r;
}
// basic_types.h:2981-2986.
inline float luminance(RGB c) { return 0.2126729f * c.r + 0.7151522f * c.g + 0.0721750f * c.b; }
inline bool all_nonneg_finite(RGB c) {
    return std::isfinite(c.r) && std::isfinite(c.g) && std::isfinite(c.b) && c.r >= 0 && c.g >= 0 &&
           c.b >= 0;
}

// common_renderer_types.h:101-125 (PCG32, XSH-RR output, 23-bit float trick).
struct Pcg32 {
    uint64_t state;
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + 1ULL;
        uint32_t xorshifted = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = static_cast<uint32_t>(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((-static_cast<int32_t>(rot)) & 31));
    }
    float uniform() {
        uint32_t bits = (next() >> 9) | 0x3f800000u;
        float f;
        std::memcpy(&f, &bits, 4);
        return f - 1.0f;
    }
};

// Jump-ahead of the PCG32 state by `delta` draws (O(log delta) LCG advance, Brown 1994 as
// used by the PCG family's pcg_advance).
inline uint64_t pcg_advance(uint64_t state, uint64_t delta) {
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

// common_renderer_types.h:1379-1405 with basic_types.h:857-864 (Duff et al. basis).
struct Frame {
    V3 t, b, n;
};
inline Frame make_frame(V3 n) {
    float sign = n.z >= 0 ? 1.0f : -1.0f;
    float a = -1 / (sign + n.z);
    float b = n.x * n.y * a;
    Frame f;
    f.t = v3(1 + sign * n.x * n.x * a, sign * b, -sign * n.x);
    f.b = v3(b, sign + n.y * n.y * a, -n.y);
    f.n = n;
    return f;
}
inline V3 to_local(const Frame& f, V3 v) { return v3(dot(f.t, v), dot(f.b, v), dot(f.n, v)); }
inline V3 from_local(const Frame& f, V3 v) {
    return v3(dot(v3(f.t.x, f.b.x, f.n.x), v), dot(v3(f.t.y, f.b.y, f.n.y), v),
              dot(v3(f.t.z, f.b.z, f.n.z), v));
}

// basic_types.h:870-874 (theta from +y, phi = atan2(-x, z) wrapped to [0, 2pi)).
inline void to_polar_yup(V3 v, float* theta, float* phi) {
    *theta = std::acos(std::min(std::max(v.y, -1.0f), 1.0f));
    *phi = std::fmod(std::atan2(-v.x, v.z) + 2 * kPi, 2 * kPi);
}
// basic_types.h:900-907.
inline V3 from_polar_yup(float phi, float theta) {
    float sp = std::sin(phi), cp = std::cos(phi);
    float st = std::sin(theta), ct = std::cos(theta);
    return v3(-sp * st, ct, cp * st);
}

// basic_types.h:1620-1628; matrix columns c0, c1, c2; M * v = (row_i . v) (:2131-2134).
struct M3 {
    V3 c0, c1, c2;
};
inline M3 quat_to_m3(const float q[4]) {
    float x = q[0], y = q[1], z = q[2], w = q[3];
    float xx = x * x, yy = y * y, zz = z * z;
    float xy = x * y, yz = y * z, zx = z * x;
    float xw = x * w, yw = y * w, zw = z * w;
    M3 m;
    m.c0 = v3(1 - 2 * (yy + zz), 2 * (xy + zw), 2 * (zx - yw));
    m.c1 = v3(2 * (xy - zw), 1 - 2 * (xx + zz), 2 * (yz + xw));
    m.c2 = v3(2 * (zx + yw), 2 * (yz - xw), 1 - 2 * (xx + yy));
    return m;
}
inline V3 mul(const M3& m, V3 v) {
    return v3(dot(v3(m.c0.x, m.c1.x, m.c2.x), v), dot(v3(m.c0.y, m.c1.y, m.c2.y), v),
              dot(v3(m.c0.z, m.c1.z, m.c2.z), v));
}

// ---------------------------------------------------------------- density grid
inline float voxel(const OrcScene& s, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || x >= s.nx || y >= s.ny || z >= s.nz) return 0.0f;
    return s.voxels[(static_cast<int64_t>(x) * s.ny + y) * s.nz + z];
}
// NanoVDB.h:1409-1414 + :2029-2032 (applyInverseMapF for a scale/translate map).
inline V3 world_to_index(const OrcScene& s, V3 p) {
    return v3((p.x - s.origin[0]) * s.inv_voxel_size, (p.y - s.origin[1]) * s.inv_voxel_size,
              (p.z - s.origin[2]) * s.inv_voxel_size);
}
// util/SampleFromVoxels.h:419-459 (first-order sampler, z then y then x lerps) and the
// float Floor at :56-65.
inline float sample_trilinear(const OrcScene& s, V3 xyz) {
    float fi = std::floor(xyz.x), fj = std::floor(xyz.y), fk = std::floor(xyz.z);
    float wx = xyz.x - fi, wy = xyz.y - fj, wz = xyz.z - fk;
    int i = static_cast<int>(fi), j = static_cast<int>(fj), k = static_cast<int>(fk);
    auto lerp = [](float a, float b, float w) { return a + w * (b - a); };
    float vz = voxel(s, i, j, k);
    float vz1 = voxel(s, i, j, k + 1);
    float vy = lerp(vz, vz1, wz);
    vz1 = voxel(s, i, j + 1, k + 1);
    vz = voxel(s, i, j + 1, k);
    float vy1 = lerp(vz, vz1, wz);
    float vx = lerp(vy, vy1, wy);
    vz = voxel(s, i + 1, j + 1, k);
    vz1 = voxel(s, i + 1, j + 1, k + 1);
    vy1 = lerp(vz, vz1, wz);
    vz1 = voxel(s, i + 1, j, k + 1);
    vz = voxel(s, i + 1, j, k);
    vy = lerp(vz, vz1, wz);
    float vx1 = lerp(vy, vy1, wy);
    return lerp(vx, vx1, wx);
}

// util/Ray.h:343-363 (slab test clipped to the ray's time span) and :512-520 (clip).
inline bool clip_ray(const float bmin[3], const float bmax[3], V3 eye, V3 dir, float tmin, float tmax,
                     float* t0o, float* t1o) {
    float inv[3] = {1 / dir.x, 1 / dir.y, 1 / dir.z};
    float e[3] = {eye.x, eye.y, eye.z};
    int sg[3] = {inv[0] < 0, inv[1] < 0, inv[2] < 0};
    auto bb = [&](int side, int axis) { return side ? bmax[axis] : bmin[axis]; };
    float t0 = (bb(sg[0], 0) - e[0]) * inv[0];
    float t2 = (bb(1 - sg[1], 1) - e[1]) * inv[1];
    if (t0 > t2) return false;
    float t1 = (bb(1 - sg[0], 0) - e[0]) * inv[0];
    float t3 = (bb(sg[1], 1) - e[1]) * inv[1];
    if (t3 > t1) return false;
    if (t3 > t0) t0 = t3;
    if (t2 < t1) t1 = t2;
    t3 = (bb(sg[2], 2) - e[2]) * inv[2];
    if (t3 > t1) return false;
    t2 = (bb(1 - sg[2], 2) - e[2]) * inv[2];
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

// ---------------------------------------------------------------- phase functions
// common_renderer_types.h:2063-2097 (Schlick); Henyey-Greenstein uses the same local
// convention (dirLocal.z = -cos(theta), theta measured from the propagation direction).
inline float phase_pdf(int kind, float g, V3 local) {
    float cos_theta = -local.z;
    if (kind == 0) {
        float d = 1 - g * cos_theta;
        return (1 - g * g) / (4 * kPi * (d * d));
    }
    float d = 1 + g * g - 2 * g * cos_theta;
    return (1 - g * g) / (4 * kPi * (d * std::sqrt(d)));
}
inline float phase_sample(int kind, float g, float u0, float u1, V3* local) {
    float cos_theta;
    if (kind == 0) {
        cos_theta = (2 * u1 + g - 1) / (2 * g * u1 - g + 1);
    } else if (std::fabs(g) < 1e-3f) {
        cos_theta = 1 - 2 * u1;
    } else {
        float sq = (1 - g * g) / (1 - g + 2 * g * u1);
        cos_theta = (1 + g * g - sq * sq) / (2 * g);
    }
    cos_theta = std::min(std::max(cos_theta, -1.0f), 1.0f);
    float phi = 2 * kPi * u0;
    float value;
    if (kind == 0) {
        float d = 1 - g * cos_theta;
        value = (1 - g * g) / (4 * kPi * (d * d));
    } else {
        float d = 1 + g * g - 2 * g * cos_theta;
        value = (1 - g * g) / (4 * kPi * (d * std::sqrt(d)));
    }
    float sin_theta = std::sqrt(1 - cos_theta * cos_theta);
    *local = v3(std::cos(phi) * sin_theta, std::sin(phi) * sin_theta, -cos_theta);
    return value;
}

// ---------------------------------------------------------------- environment
inline int env_texel_x(const OrcScene& s, float u) {
    int x = static_cast<int>(u * s.env_w);
    return std::min(std::max(x, 0), s.env_w - 1);
}
inline int env_texel_y(const OrcScene& s, float v) {
    int y = static_cast<int>(v * s.env_h);
    return std::min(std::max(y, 0), s.env_h - 1);
}
inline RGB env_texel(const OrcScene& s, int x, int y) {
    const float* p = s.env_rgb + 3 * (static_cast<int64_t>(y) * s.env_w + x);
    return rgb(p[0], p[1], p[2]);
}
inline float mip_texel(const OrcScene& s, int level, int x, int y) {
    int w = std::max(s.map_w >> level, 1);
    return s.imp_mips[s.imp_offsets[level] + static_cast<int64_t>(y) * w + x];
}

// common_renderer_types.h:479-548 (hierarchical mip walk from the 2x2 (or 2x1) level down).
inline void imp_sample(const OrcScene& s, float u0, float u1, int* px, int* py, float* ru0,
                       float* ru1, float* prob) {
    int ix = 0, iy = 0;
    *prob = 1;
    int cur_w = 2, cur_h = s.map_w > s.map_h ? 1 : 2;
    for (int level = s.num_mips - 2; level >= 0; --level) {
        ix *= 2;
        iy *= 2;
        // Bounds tests as in the reference: texel centre + offset compared with the level's dims.
        bool has_lower = (iy + 1.5f) < cur_h;
        bool has_right = (ix + 1.5f) < cur_w;
        float vul = mip_texel(s, level, ix, iy);
        float vur = has_right ? mip_texel(s, level, ix + 1, iy) : 0.0f;
        float vll = has_lower ? mip_texel(s, level, ix, iy + 1) : 0.0f;
        float vlr = (has_right && has_lower) ? mip_texel(s, level, ix + 1, iy + 1) : 0.0f;
        float left = vll + vul;
        float right = vlr + vur;
        u0 *= (left + right);
        *prob *= 1.0f / (left + right);
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
            *prob *= upper;
            u1 = (u1 - 0) / upper;
        } else {
            iy += 1;
            *prob *= lower;
            u1 = (u1 - upper) / lower;
        }
        ix = std::min(ix, cur_w - 1);
        iy = std::min(iy, cur_h - 1);
        cur_w *= 2;
        cur_h *= 2;
    }
    *px = ix;
    *py = iy;
    *ru0 = u0;
    *ru1 = u1;
}

// common_renderer_types.h:2419-2440 + :987-1000 (sample then rotate, power coefficient).
inline RGB env_sample(const OrcScene& s, float u0, float u1, V3* dir, float* dir_pdf) {
    float prob;
    int px, py;
    imp_sample(s, u0, u1, &px, &py, &u0, &u1, &prob);
    float u = (px + u0) / s.env_w;
    float v = (py + u1) / s.env_h;
    float uv_pdf = static_cast<float>(static_cast<uint32_t>(s.env_w) * static_cast<uint32_t>(s.env_h)) * prob;
    float phi = 2 * kPi * u;
    float theta = kPi * v;
    *dir_pdf = uv_pdf / (2 * (kPi * kPi) * std::sin(theta));
    RGB radiance;
    if (!std::isfinite(*dir_pdf)) {
        *dir_pdf = 0.0f;
        radiance = rgb(0, 0, 0);
    } else {
        radiance = env_texel(s, env_texel_x(s, u), env_texel_y(s, v));
    }
    radiance = s.env_power * radiance;
    float pos_phi = phi - s.env_rotation;
    pos_phi = pos_phi - std::floor(pos_phi / (2 * kPi)) * 2 * kPi;
    *dir = from_polar_yup(pos_phi, theta);
    return radiance;
}

// common_renderer_types.h:2442-2458 + :1002-1013.
inline RGB env_evaluate(const OrcScene& s, V3 dir, float* hyp_pdf) {
    float theta, pos_phi;
    to_polar_yup(dir, &theta, &pos_phi);
    float phi = pos_phi + s.env_rotation;
    phi = phi - std::floor(phi / (2 * kPi)) * 2 * kPi;
    float u = phi / (2 * kPi), v = theta / kPi;
    int tx = env_texel_x(s, u), ty = env_texel_y(s, v);
    RGB radiance = env_texel(s, tx, ty);
    float prob = mip_texel(s, 0, tx, ty) / s.imp_integral;
    float uv_pdf = static_cast<float>(static_cast<uint32_t>(s.env_w) * static_cast<uint32_t>(s.env_h)) * prob;
    *hyp_pdf = uv_pdf / (2 * (kPi * kPi) * std::sin(theta));
    if (!std::isfinite(*hyp_pdf)) {
        *hyp_pdf = 0.0f;
        radiance = rgb(0, 0, 0);
    }
    return s.env_power * radiance;
}

// ---------------------------------------------------------------- tracking
// Limits applied when the configurable caps are disabled (same values as the device tracker).
constexpr uint32_t kHardStepCap = 1u << 24;
constexpr uint32_t kHardVertexCap = 1u << 16;
inline uint32_t step_cap(const OrcScene& s) {
    return s.max_steps > 0 ? static_cast<uint32_t>(s.max_steps) : kHardStepCap;
}
// Result of tracking one segment.
enum SegEnd { SEG_EXIT = 0, SEG_COLLIDE = 1, SEG_CAP = 2 };

struct Counters {
    int64_t lookups = 0;
    uint32_t primary = 0, shadow = 0;
};

inline float density_at(const OrcScene& s, V3 eye, V3 dir, float t) {
    V3 p = eye + dir * t;
    return s.density_coeff * sample_trilinear(s, world_to_index(s, p));
}

// Majorant-grid DDA in index space (8^3-voxel cells). Shared definition with the device
// tracker: overshooting a cell boundary restarts sampling at the boundary (memoryless).
struct Dda {
    int cell[3];
    int step[3];
    float tnext[3], tdelta[3];
};
inline void dda_init(const OrcScene& s, V3 eye, V3 dir, float t, Dda* d) {
    float o[3] = {(eye.x - s.origin[0]) * s.inv_voxel_size, (eye.y - s.origin[1]) * s.inv_voxel_size,
                  (eye.z - s.origin[2]) * s.inv_voxel_size};
    float dd[3] = {dir.x * s.inv_voxel_size, dir.y * s.inv_voxel_size, dir.z * s.inv_voxel_size};
    int cdim[3] = {s.cx, s.cy, s.cz};
    const float size = static_cast<float>(1 << (s.maj_shift < 3 ? 3 : s.maj_shift));
    const float inv_size = 1.0f / size;
    for (int a = 0; a < 3; ++a) {
        float p = o[a] + dd[a] * t;
        int c = static_cast<int>(std::floor(p * inv_size));
        c = std::min(std::max(c, 0), cdim[a] - 1);
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

// Russian roulette on a shadow ray's visibility once it drops below s.shadow_rr (configuration
// mode; an extra draw from the path's stream). Returns true when the ray is terminated (vis = 0).
inline bool shadow_roulette(const OrcScene& s, Pcg32& rng, float* vis) {
    if (!(*vis < s.shadow_rr)) return false;
    const float q = *vis / s.shadow_rr;
    if (rng.uniform() >= q) {
        *vis = 0.0f;
        return true;
    }
    *vis = s.shadow_rr;
    return false;
}

// Tracks [t, t1] along (eye, dir). Delta tracking (shadow = false) returns SEG_COLLIDE with
// *t at the collision; ratio tracking (shadow = true) multiplies *vis.
inline SegEnd track(const OrcScene& s, Pcg32& rng, V3 eye, V3 dir, float* tio, float t1, bool shadow,
                    float* vis, uint32_t* steps, int64_t* lookups) {
    float t = *tio;
    uint32_t seg_steps = 0;
    if (s.majorant_mode == 0) {
        // optix_pathtracing_kernels.cu:111-124 and renderer_kernel_common.h:372-381.
        const float maj = s.density_coeff * s.global_majorant;
        while (true) {
            t += -std::log(1.0f - rng.uniform()) / maj;
            if (!(t <= t1)) break;  // also ends the segment on a NaN distance
            float density = density_at(s, eye, dir, t);
            ++*steps;
            ++*lookups;
            ++seg_steps;
            if (shadow) {
                *vis *= (1 - density / maj);
                if (shadow_roulette(s, rng, vis)) {
                    *tio = t;
                    return SEG_EXIT;
                }
            } else if (rng.uniform() < density / maj) {
                *tio = t;
                return SEG_COLLIDE;
            }
            if (seg_steps >= step_cap(s)) return SEG_CAP;
        }
        *tio = t;
        return SEG_EXIT;
    }
    Dda d;
    dda_init(s, eye, dir, t, &d);
    while (true) {
        float texit = std::min(std::min(d.tnext[0], d.tnext[1]), std::min(d.tnext[2], t1));
        int64_t ci = (static_cast<int64_t>(d.cell[0]) * s.cy + d.cell[1]) * s.cz + d.cell[2];
        float maj = s.density_coeff * s.cell_majorant[ci];
        if (maj > 0) {
            while (true) {
                float tt = t + -std::log(1.0f - rng.uniform()) / maj;
                if (tt >= texit) break;
                t = tt;
                float density = density_at(s, eye, dir, t);
                ++*steps;
                ++*lookups;
                ++seg_steps;
                if (shadow) {
                    *vis *= (1 - density / maj);
                    if (shadow_roulette(s, rng, vis)) {
                        *tio = t1;
                        return SEG_EXIT;
                    }
                } else if (rng.uniform() < density / maj) {
                    *tio = t;
                    return SEG_COLLIDE;
                }
                if (seg_steps >= step_cap(s)) return SEG_CAP;
            }
        }
        t = texit;
        if (texit >= t1) break;
        int a = (d.tnext[0] <= d.tnext[1] && d.tnext[0] <= d.tnext[2]) ? 0 : (d.tnext[1] <= d.tnext[2] ? 1 : 2);
        d.cell[a] += d.step[a];
        int cdim[3] = {s.cx, s.cy, s.cz};
        if (d.cell[a] < 0 || d.cell[a] >= cdim[a]) break;
        d.tnext[a] += d.tdelta[a];
    }
    *tio = t1;
    return SEG_EXIT;
}

// renderer_kernel_common.h:297-403 restricted to the environment light, plus the
// directional sun of the config mode (picked with probability sun_prob, no MIS: delta light).
inline RGB next_event(const OrcScene& s, Pcg32& rng, V3 pos, const Frame& fr, float* shadow_vis_out,
                      uint32_t* shadow_steps, int64_t* lookups, bool* capped) {
    float u_light = rng.uniform();
    float u0 = rng.uniform();
    float u1 = rng.uniform();
    bool pick_sun = false;
    float light_prob = 1.0f;
    if (s.sun_enabled && s.env_enabled) {
        if (u_light < s.sun_prob) {
            pick_sun = true;
            light_prob = s.sun_prob;
        } else {
            light_prob = 1.0f - s.sun_prob;
        }
    } else if (s.sun_enabled) {
        pick_sun = true;
    } else if (!s.env_enabled) {
        return rgb(0, 0, 0);
    }

    V3 light_dir;
    RGB emittance;
    float area_pdf;
    if (pick_sun) {
        light_dir = v3(s.sun_dir[0], s.sun_dir[1], s.sun_dir[2]);
        emittance = rgb(s.sun_irradiance[0], s.sun_irradiance[1], s.sun_irradiance[2]);
        area_pdf = light_prob;
    } else {
        float dir_pdf;
        RGB radiance = env_sample(s, u0, u1, &light_dir, &dir_pdf);
        emittance = kPi * radiance;
        area_pdf = dir_pdf;
        if (area_pdf == 0.0f) return rgb(0, 0, 0);
        area_pdf *= light_prob;
    }
    V3 shadow_dir = -light_dir;
    V3 light_normal = -light_dir;
    float lp_cos = dot(shadow_dir, light_normal);
    if (lp_cos <= 0.0f) return rgb(0, 0, 0);
    float trace_len = 2 * s.world_radius;
    V3 light_point = pos + trace_len * -shadow_dir;

    float vis = 1.0f;
    float t0, t1;
    if (clip_ray(s.bbox_min, s.bbox_max, light_point, shadow_dir, 0.0f, trace_len, &t0, &t1)) {
        float t = std::fmax(0.0f, t0);
        if (track(s, rng, light_point, shadow_dir, &t, t1, true, &vis, shadow_steps, lookups) == SEG_CAP) {
            *capped = true;
            return rgb(0, 0, 0);
        }
    }
    *shadow_vis_out = vis;
    RGB ret = rgb(0, 0, 0);
    if (vis > 0.0f) {
        V3 v_in_local = to_local(fr, -shadow_dir);
        float pf = phase_pdf(s.phase_kind, s.phase_param, v_in_local);
        RGB fs = rgb(s.albedo, s.albedo, s.albedo) * pf;
        if (pick_sun) {
            ret = fs * emittance * (vis / area_pdf);
        } else {
            float bsdf_pdf = pf * lp_cos / 1.0f;
            if (!std::isfinite(bsdf_pdf)) bsdf_pdf = 0.0f;
            float light_pdf = area_pdf;
            float mis = (light_pdf * light_pdf) / ((bsdf_pdf * bsdf_pdf) + (light_pdf * light_pdf));
            RGB le = div(emittance, kPi);
            float g = lp_cos * 1.0f / 1.0f;
            ret = fs * le * (vis * mis * g / area_pdf);
        }
    }
    return ret;
}

}  // namespace

// ------------------------------------------------------------------------------ surfaces
// The reference's surface path (renderer_kernel_common.h:72-403, common_renderer_types.h:
// 1265-1307, 1483-1985, compute_light_probs.cu:19-157) restated over prepared world triangles.
struct OrcSurfaces {
    struct Mat {
        int kind;
        float diffuse[3], specular[3], roughness;
        float emit[3];
        bool emissive;
    };
    struct Inst {
        float m[12], nm[9];
        float uniform_scale;
        uint32_t first_geom, num_geoms, first_world_tri_of_geom0;
        std::vector<float> group_w, group_cdf;
        float group_integral;
    };
    struct Geom {
        uint32_t num_tris, material;
        std::vector<float> w, cdf;
        float integral;
        std::vector<float> nrm, tan;   // object space, 3 per vertex
        std::vector<uint32_t> tri;     // 3 per triangle
    };
    std::vector<Mat> mats;
    std::vector<Geom> geoms;
    std::vector<Inst> insts;
    std::vector<float> inst_w, inst_cdf;
    float inst_integral = 0;
    // World triangles: 9 floats each, and their (instance, geometry, primitive).
    std::vector<float> pos;
    std::vector<uint32_t> owner_inst, owner_geom, owner_prim;
    std::vector<uint32_t> inst_geom_first_tri;   // per (instance, geometry of its group): first world triangle
};

namespace {

float orc_unorm8(float v) {
    const float sc = 255.0f * v;
    const uint32_t q = std::min<uint32_t>(sc > 0.0f ? static_cast<uint32_t>(sc) : 0u, 255u);
    return static_cast<float>(q);
}
// sRGB decode of an 8-bit immediate texel (renderer_scene.cpp:1171-1200 read mode NormalizedFloat_sRGB).
float orc_srgb8(float v) {
    const double c = orc_unorm8(v) / 255.0;
    return static_cast<float>(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
}

// The BSDF parameters setupBSDFBody derives from a material's immediate textures
// (common_renderer_types.h:1524-1541 Lambert; 1924-1933 and 1962-1985 SimplePBR with
// reflectance 0.5 and smoothness min(1 - roughness, 0.999)).
OrcSurfaces::Mat decode_material(const OrcSurfMaterial& m) {
    OrcSurfaces::Mat d{};
    d.kind = m.kind;
    float base[3];
    for (int a = 0; a < 3; ++a) base[a] = orc_srgb8(m.base_color[a]);
    if (m.kind == 1) {
        for (int a = 0; a < 3; ++a) {
            d.diffuse[a] = base[a];
            d.specular[a] = 0.0f;
        }
        d.roughness = 1.0f;
    } else {
        const float rough = orc_unorm8(m.roughness) / 255.0f, metal = orc_unorm8(m.metallic) / 255.0f;
        const float smooth = std::min(1.0f - rough, 0.999f);
        for (int a = 0; a < 3; ++a) {
            d.diffuse[a] = base[a] * (1 - metal);
            d.specular[a] = 0.16f * (0.5f * 0.5f) * (1 - metal) + base[a] * metal;
        }
        d.roughness = 1 - smooth;
    }
    d.emissive = m.emittance[0] != 0.0f || m.emittance[1] != 0.0f || m.emittance[2] != 0.0f;
    for (int a = 0; a < 3; ++a) d.emit[a] = m.emittance[a];
    return d;
}

V3 cross3(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

float excl_cdf(const std::vector<float>& w, std::vector<float>* cdf) {
    cdf->resize(w.size());
    float acc = 0.0f;
    for (size_t i = 0; i < w.size(); ++i) {
        (*cdf)[i] = acc;
        acc = acc + w[i];
    }
    return w.empty() ? 0.0f : (*cdf)[w.size() - 1] + w.back();
}

// DiscreteDistribution1D::sample (common_renderer_types.h:165-188).
uint32_t dist_sample(const std::vector<float>& w, const std::vector<float>& cdf, float integral, float u, float* prob,
                     float* remapped) {
    const uint32_t n = static_cast<uint32_t>(w.size());
    u *= integral;
    int idx = 0;
    uint32_t p2 = 1;
    while (p2 < n) p2 <<= 1;
    for (int d = static_cast<int>(p2 >> 1); d >= 1; d >>= 1) {
        if (idx + d >= static_cast<int>(n)) continue;
        if (cdf[idx + d] <= u) idx += d;
    }
    const float lc = cdf[idx];
    const float rc = idx < static_cast<int>(n) - 1 ? cdf[idx + 1] : integral;
    *remapped = (u - lc) / (rc - lc);
    *prob = w[idx] / integral;
    return static_cast<uint32_t>(idx);
}

V3 xf_point(const float* m, const float* p) {
    return v3(m[0] * p[0] + m[1] * p[1] + m[2] * p[2] + m[3] * 1.0f, m[4] * p[0] + m[5] * p[1] + m[6] * p[2] + m[7] * 1.0f,
              m[8] * p[0] + m[9] * p[1] + m[10] * p[2] + m[11] * 1.0f);
}
V3 xf_vector(const float* m, V3 v) {
    return v3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z, m[8] * v.x + m[9] * v.y + m[10] * v.z);
}
V3 xf_normal(const float* nm, V3 n) {
    return v3(nm[0] * n.x + nm[1] * n.y + nm[2] * n.z, nm[3] * n.x + nm[4] * n.y + nm[5] * n.z,
              nm[6] * n.x + nm[7] * n.y + nm[8] * n.z);
}
V3 tri_vertex(const OrcSurfaces& S, uint32_t t, int k) {
    const float* q = &S.pos[9 * static_cast<size_t>(t) + 3 * k];
    return v3(q[0], q[1], q[2]);
}

// Möller-Trumbore in the order of renderer_kernel_common.h:236-248; two-sided, t in [tmin, tmax].
bool tri_hit(V3 o, V3 d, V3 p0, V3 p1, V3 p2, float tmin, float tmax, float* t, float* b1, float* b2) {
    const V3 e1 = p1 - p0, e2 = p2 - p0;
    const V3 pv = cross3(d, e2);
    const float det = dot(e1, pv);
    if (det == 0.0f) return false;
    const float rdet = 1.0f / det;
    const V3 tv = o - p0;
    const float u = dot(tv, pv) * rdet;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    const V3 qv = cross3(tv, e1);
    const float v = dot(d, qv) * rdet;
    if (!(v >= 0.0f && u + v <= 1.0f)) return false;
    const float tt = dot(e2, qv) * rdet;
    if (!(tt >= tmin && tt <= tmax)) return false;
    *t = tt;
    *b1 = u;
    *b2 = v;
    return true;
}

// Closest triangle by exhaustive search; equal distances go to the lower triangle index.
int32_t closest_hit(const OrcSurfaces& S, V3 o, V3 d, float tmax, float* tout, float* b1o, float* b2o) {
    int32_t best = -1;
    float bt = tmax;
    const uint32_t n = static_cast<uint32_t>(S.owner_inst.size());
    for (uint32_t t = 0; t < n; ++t) {
        float tt, b1, b2;
        if (tri_hit(o, d, tri_vertex(S, t, 0), tri_vertex(S, t, 1), tri_vertex(S, t, 2), 0.0f, bt, &tt, &b1, &b2) &&
            (best < 0 || tt < bt)) {
            best = static_cast<int32_t>(t);
            bt = tt;
            *b1o = b1;
            *b2o = b2;
        }
    }
    *tout = bt;
    return best;
}

bool any_hit(const OrcSurfaces& S, V3 o, V3 d, float tmax) {
    const uint32_t n = static_cast<uint32_t>(S.owner_inst.size());
    for (uint32_t t = 0; t < n; ++t) {
        float tt, b1, b2;
        if (tri_hit(o, d, tri_vertex(S, t, 0), tri_vertex(S, t, 1), tri_vertex(S, t, 2), 0.0f, tmax, &tt, &b1, &b2))
            return true;
    }
    return false;
}

struct SurfPt {
    V3 pos, gn;
    Frame sf;
    float hyp_area_pdf;
    uint32_t material;
};

// computeSurfacePoint (renderer_kernel_common.h:72-124).
SurfPt surface_point(const OrcSurfaces& S, uint32_t tri, float b1, float b2, bool env_enabled) {
    const OrcSurfaces::Inst& in = S.insts[S.owner_inst[tri]];
    const OrcSurfaces::Geom& ge = S.geoms[S.owner_geom[tri]];
    const uint32_t prim = S.owner_prim[tri];
    const V3 p0 = tri_vertex(S, tri, 0), p1 = tri_vertex(S, tri, 1), p2 = tri_vertex(S, tri, 2);
    const float b0 = 1 - (b1 + b2);
    SurfPt sp;
    sp.pos = b0 * p0 + b1 * p1 + b2 * p2;
    const V3 gn = cross3(p1 - p0, p2 - p0);
    const float area = 0.5f * std::sqrt(gn.x * gn.x + gn.y * gn.y + gn.z * gn.z);
    sp.gn = gn * (1.0f / (2 * area));
    const uint32_t* vi = &ge.tri[3 * static_cast<size_t>(prim)];
    auto at = [](const std::vector<float>& a, uint32_t k) { return v3(a[3 * k], a[3 * k + 1], a[3 * k + 2]); };
    const V3 ln = b0 * at(ge.nrm, vi[0]) + b1 * at(ge.nrm, vi[1]) + b2 * at(ge.nrm, vi[2]);
    const V3 lt = b0 * at(ge.tan, vi[0]) + b1 * at(ge.tan, vi[1]) + b2 * at(ge.tan, vi[2]);
    sp.sf.n = normalize(xf_normal(in.nm, ln));
    sp.sf.t = normalize(xf_vector(in.m, lt));
    sp.sf.b = cross3(sp.sf.n, sp.sf.t);
    sp.material = ge.material;
    float light_prob = 1.0f;
    if (env_enabled) light_prob *= (1 - 0.25f);
    const float inst_imp = (in.uniform_scale * in.uniform_scale) * in.group_integral;
    sp.hyp_area_pdf = 0.0f;
    if (S.inst_integral > 0.0f) {
        const float inst_prob = inst_imp / S.inst_integral;
        if (inst_prob != 0.0f) {
            light_prob *= inst_prob;
            const float geom_prob = ge.integral / in.group_integral;
            if (geom_prob != 0.0f) {
                light_prob *= geom_prob;
                light_prob *= ge.integral == 0.0f ? 0.0f : ge.w[prim] / ge.integral;
                sp.hyp_area_pdf = light_prob / area;
            }
        }
    }
    return sp;
}

// cosineSampleHemisphere over concentricSampleDisk (common_renderer_types.h:1265-1307).
V3 cos_hemisphere(float u0, float u1) {
    const float sx = 2 * u0 - 1, sy = 2 * u1 - 1;
    float x = 0.0f, y = 0.0f;
    if (!(sx == 0 && sy == 0)) {
        float r, th;
        if (sx >= -sy) {
            if (sx > sy) {
                r = sx;
                th = sy / sx;
            } else {
                r = sy;
                th = 2 - sx / sy;
            }
        } else if (sx > sy) {
            r = -sy;
            th = 6 + sx / sy;
        } else {
            r = -sx;
            th = 4 + sy / sx;
        }
        th *= kPi / 4;
        x = r * std::cos(th);
        y = r * std::sin(th);
    }
    return v3(x, y, std::sqrt(std::fmax(0.0f, 1.0f - x * x - y * y)));
}

inline float p5(float x) {
    const float x2 = x * x;
    return x * (x2 * x2);
}
inline float lerp1(float a, float b, float t) { return (1 - t) * a + t * b; }

// GGX of the dichromatic BRDF (common_renderer_types.h:1595-1650).
float g_d(float ag, V3 m) {
    if (m.z <= 0.0f) return 0.0f;
    const float tmp = m.x * m.x + m.y * m.y + (m.z * ag) * (m.z * ag);
    return (ag * ag) / (kPi * (tmp * tmp));
}
float g_g1(float ag, V3 v, V3 m) {
    if (dot(v, m) * v.z <= 0) return 0.0f;
    const float tmp = (ag * ag) * (v.x * v.x + v.y * v.y) / (v.z * v.z);
    return 2 / (1 + std::sqrt(1 + tmp));
}
float g_hc(float ag, V3 v1, V3 v2, V3 m) {
    const float a1 = (ag * ag) * (v1.x * v1.x + v1.y * v1.y) / (v1.z * v1.z);
    const float a2 = (ag * ag) * (v2.x * v2.x + v2.y * v2.y) / (v2.z * v2.z);
    const float l1 = (-1 + std::sqrt(1 + a1)) / 2;
    const float l2 = (-1 + std::sqrt(1 + a2)) / 2;
    const float c1 = (dot(v1, m) / v1.z) > 0 ? 1.0f : 0.0f;
    const float c2 = (dot(v2, m) / v2.z) > 0 ? 1.0f : 0.0f;
    return c1 * c2 / (1 + l1 + l2);
}
float g_pdf(float ag, V3 v, V3 m) { return g_g1(ag, v, m) * std::fabs(dot(v, m)) * g_d(ag, m) / std::fabs(v.z); }
float g_sample(float ag, V3 v, float u0, float u1, V3* m, float* mpdf) {
    const V3 sv = normalize(v3(ag * v.x, ag * v.y, v.z));
    const float d2 = std::sqrt(sv.x * sv.x + sv.y * sv.y);
    const float rd = 1.0f / d2;
    const V3 T1 = (sv.z < 0.9999f) ? v3(sv.y * rd, -sv.x * rd, 0) : v3(1, 0, 0);
    const V3 T2 = v3(T1.y * sv.z, -T1.x * sv.z, d2);
    const float a = 1.0f / (1.0f + sv.z);
    const float r = std::sqrt(u0);
    const float phi = kPi * ((u1 < a) ? u1 / a : 1 + (u1 - a) / (1.0f - a));
    const float sp = std::sin(phi), cp = std::cos(phi);
    const float P1 = r * cp;
    const float P2 = r * sp * ((u1 < a) ? 1.0f : sv.z);
    V3 mm = P1 * T1 + P2 * T2 + std::sqrt(1.0f - P1 * P1 - P2 * P2) * sv;
    mm = normalize(v3(ag * mm.x, ag * mm.y, mm.z));
    *m = mm;
    const float D = g_d(ag, mm);
    *mpdf = g_g1(ag, v, mm) * std::fabs(dot(v, mm)) * D / std::fabs(v.z);
    return D;
}

struct Brdf {
    RGB diff, spec;
    float rough;
    int kind;
};
Brdf brdf_of(const OrcSurfaces::Mat& m) {
    return Brdf{rgb(m.diffuse[0], m.diffuse[1], m.diffuse[2]), rgb(m.specular[0], m.specular[1], m.specular[2]), m.roughness,
                m.kind};
}
// Lobe selection weights (:1690-1705, non-fitted).
void lobe_weights(const Brdf& f, float qz, float vz, float* wd, float* ws) {
    const float vn5 = p5(1 - vz);
    const float fd90 = 0.5f * f.rough + 2 * f.rough * qz * qz;
    const float edf = lerp1(1.0f, fd90, vn5);
    *wd = luminance(f.diff) * (edf * edf) * lerp1(1.0f, 1.0f / 1.51f, f.rough);
    *ws = lerp1(luminance(f.spec), 1.0f, p5(1 - vz));
}
RGB dichro_value(const Brdf& f, float ag, V3 L, V3 V, V3 m, float lh, float D) {
    const float G = g_hc(ag, L, V, m);
    const float w = p5(1 - lh);
    const RGB F = (1 - w) * f.spec + w * rgb(1.0f, 1.0f, 1.0f);
    RGB spec = F * ((D * G) / (4 * L.z * V.z));
    if (G == 0) spec = rgb(0, 0, 0);
    const float fd90 = 0.5f * f.rough + 2 * f.rough * lh * lh;
    const float fo = lerp1(1.0f, fd90, p5(1 - V.z));
    const float fi = lerp1(1.0f, fd90, p5(1 - L.z));
    return f.diff * (fo * fi * lerp1(1.0f, 1.0f / 1.51f, f.rough) / kPi) + spec;
}
// sampleF (Lambert :1497-1505, dichromatic :1680-1790).
RGB brdf_sample(const Brdf& f, V3 q, float u0, float u1, V3* out, float* pdf) {
    if (f.kind == 1) {
        V3 d = cos_hemisphere(u0, u1);
        *pdf = d.z / kPi;
        if (q.z <= 0.0f) d.z *= -1;
        *out = d;
        return div(f.diff, kPi);
    }
    const float ag = f.rough * f.rough;
    const bool entering = q.z >= 0.0f;
    const V3 V = entering ? q : -q;
    float wd, ws;
    lobe_weights(f, q.z, V.z, &wd, &ws);
    const float sum = wd + ws;
    if (sum == 0.0f) {
        *pdf = 0.0f;
        return rgb(0, 0, 0);
    }
    float pd, ps, lh, D;
    V3 L, m;
    if (sum * u1 < wd) {
        const float ud1 = (sum * u1 - 0) / wd;
        L = cos_hemisphere(u0, ud1);
        pd = L.z / kPi;
        m = normalize(L + V);
        lh = std::fmin(dot(L, m), 1.0f);
        ps = (1.0f / (4 * lh)) * g_pdf(ag, V, m);
        D = g_d(ag, m);
    } else {
        const float ud1 = (sum * u1 - wd) / ws;
        float mp;
        D = g_sample(ag, V, u0, ud1, &m, &mp);
        const float vh = std::fmin(dot(V, m), 1.0f);
        lh = vh;
        L = (2 * vh) * m - V;
        if (L.z * V.z <= 0) {
            *pdf = 0.0f;
            return rgb(0, 0, 0);
        }
        ps = (1.0f / (4 * lh)) * mp;
        pd = L.z / kPi;
    }
    const RGB val = dichro_value(f, ag, L, V, m, lh, D);
    *out = entering ? L : -L;
    *pdf = (pd * wd + ps * ws) / sum;
    return val;
}
// evaluateF and evaluatePDF (Lambert :1506-1517, dichromatic :1792-1875).
RGB brdf_eval(const Brdf& f, V3 q, V3 s) {
    if (f.kind == 1) return (q.z * s.z > 0) ? div(f.diff, kPi) : rgb(0, 0, 0);
    if (s.z * q.z <= 0) return rgb(0, 0, 0);
    const float ag = f.rough * f.rough;
    const bool entering = q.z >= 0.0f;
    const V3 V = entering ? q : -q, L = entering ? s : -s;
    const V3 m = normalize(L + V);
    return dichro_value(f, ag, L, V, m, dot(L, m), g_d(ag, m));
}
float brdf_pdf(const Brdf& f, V3 q, V3 s) {
    if (f.kind == 1) return (q.z * s.z > 0) ? std::fabs(s.z) / kPi : 0.0f;
    const float ag = f.rough * f.rough;
    const bool entering = q.z >= 0.0f;
    const V3 V = entering ? q : -q, L = entering ? s : -s;
    const V3 m = normalize(L + V);
    const float common = 1.0f / (4 * dot(L, m));
    float wd, ws;
    lobe_weights(f, q.z, V.z, &wd, &ws);
    const float sum = wd + ws;
    if (sum == 0.0f) return 0.0f;
    return ((L.z / kPi) * wd + (common * g_pdf(ag, V, m)) * ws) / sum;
}

// offsetRayOrigin (common_renderer_types.h:1324-1349).
float offset1(float p, float n) {
    const int32_t oi = static_cast<int32_t>(256.0f * n);
    int32_t bits;
    std::memcpy(&bits, &p, 4);
    bits += (p < 0 ? -oi : oi);
    float p1;
    std::memcpy(&p1, &bits, 4);
    const float p2 = p + (1.0f / 65536.0f) * n;
    return std::fabs(p) < (1.0f / 32.0f) ? p2 : p1;
}
V3 offset_origin(V3 p, V3 n) { return v3(offset1(p.x, n.x), offset1(p.y, n.y), offset1(p.z, n.z)); }

// sampleLight<false> over the emitting triangles (renderer_kernel_common.h:146-290).
bool sample_area(const OrcSurfaces& S, float ul, float u0, float u1, V3* pos, V3* nrm, RGB* emit, float* area_pdf) {
    float light_prob = 1.0f;
    float inst_prob, ug;
    const uint32_t ii = dist_sample(S.inst_w, S.inst_cdf, S.inst_integral, ul, &inst_prob, &ug);
    light_prob *= inst_prob;
    if (inst_prob == 0.0f) return false;
    const OrcSurfaces::Inst& in = S.insts[ii];
    float geom_prob, up;
    const uint32_t gi = dist_sample(in.group_w, in.group_cdf, in.group_integral, ug, &geom_prob, &up);
    light_prob *= geom_prob;
    if (geom_prob == 0.0f) return false;
    const OrcSurfaces::Geom& ge = S.geoms[in.first_geom + gi];
    float prim_prob, unused;
    const uint32_t prim = dist_sample(ge.w, ge.cdf, ge.integral, up, &prim_prob, &unused);
    light_prob *= prim_prob;
    const uint32_t tri = S.inst_geom_first_tri[in.first_world_tri_of_geom0 + gi] + prim;
    const V3 p0 = tri_vertex(S, tri, 0), p1 = tri_vertex(S, tri, 1), p2 = tri_vertex(S, tri, 2);
    const V3 gnv = cross3(p1 - p0, p2 - p0);
    float t0 = 0.5f * u0, t1 = 0.5f * u1;
    const float off = t1 - t0;
    if (off > 0)
        t1 += off;
    else
        t0 -= off;
    const float t2 = 1 - (t0 + t1);
    *area_pdf = light_prob * (2.0f / std::sqrt(gnv.x * gnv.x + gnv.y * gnv.y + gnv.z * gnv.z));
    *pos = t0 * p0 + t1 * p1 + t2 * p2;
    const uint32_t* vi = &ge.tri[3 * static_cast<size_t>(prim)];
    auto at = [](const std::vector<float>& a, uint32_t k) { return v3(a[3 * k], a[3 * k + 1], a[3 * k + 2]); };
    *nrm = normalize(xf_normal(in.nm, t0 * at(ge.nrm, vi[0]) + t1 * at(ge.nrm, vi[1]) + t2 * at(ge.nrm, vi[2])));
    const OrcSurfaces::Mat& mt = S.mats[ge.material];
    *emit = mt.emissive ? rgb(mt.emit[0], mt.emit[1], mt.emit[2]) : rgb(0, 0, 0);
    return true;
}

// performNextEventEstimation (renderer_kernel_common.h:297-403) in a scene with surfaces: the
// environment (with the sun of the configuration mode) against the emitting triangles with
// probToSampleEnvLight, triangle visibility, then ratio tracking through the volume. At a
// medium vertex `surf` is null and `fr` is the phase frame; at a surface vertex `surf` holds the
// point and `f`, `q` its BSDF and query direction.
RGB next_event_surf(const OrcScene& s, Pcg32& rng, V3 pos, const Frame& fr, const SurfPt* surf, const Brdf* f, V3 q,
                    uint32_t* shadow_steps, int64_t* lookups, bool* capped) {
    const OrcSurfaces& S = *s.surfaces;
    float u_light = rng.uniform();
    const float u0 = rng.uniform();
    const float u1 = rng.uniform();
    const bool areas = S.inst_integral > 0.0f;
    const bool env_group = s.env_enabled || s.sun_enabled;
    if (!env_group && !areas) return rgb(0, 0, 0);
    bool select_env = false;
    float type_prob = 1.0f;
    if (env_group) {
        if (areas) {
            if (u_light < 0.25f) {
                type_prob = 0.25f;
                u_light /= type_prob;
                select_env = true;
            } else {
                type_prob = 1.0f - 0.25f;
                u_light = (u_light - 0.25f) / type_prob;
            }
        } else {
            select_env = true;
        }
    }
    bool pick_sun = false;
    RGB emittance;
    float area_pdf, lp_cos, dist2 = 1.0f, trace_length = 2 * s.world_radius;
    V3 light_point, sdir;
    if (select_env) {
        float light_prob = 1.0f;
        if (s.sun_enabled && s.env_enabled) {
            if (u_light < s.sun_prob) {
                pick_sun = true;
                light_prob = s.sun_prob;
            } else {
                light_prob = 1.0f - s.sun_prob;
            }
        } else if (s.sun_enabled) {
            pick_sun = true;
        }
        V3 light_dir;
        if (pick_sun) {
            light_dir = v3(s.sun_dir[0], s.sun_dir[1], s.sun_dir[2]);
            emittance = rgb(s.sun_irradiance[0], s.sun_irradiance[1], s.sun_irradiance[2]);
            area_pdf = light_prob;
        } else {
            float dp;
            const RGB radiance = env_sample(s, u0, u1, &light_dir, &dp);
            emittance = kPi * radiance;
            area_pdf = dp;
            if (area_pdf == 0.0f) return rgb(0, 0, 0);
            area_pdf *= light_prob;
        }
        area_pdf *= type_prob;
        sdir = -light_dir;
        lp_cos = dot(sdir, -light_dir);
        if (lp_cos <= 0.0f) return rgb(0, 0, 0);
        light_point = pos + trace_length * light_dir;
    } else {
        V3 lp, ln;
        if (!sample_area(S, u_light, u0, u1, &lp, &ln, &emittance, &area_pdf)) return rgb(0, 0, 0);
        if (area_pdf == 0.0f) return rgb(0, 0, 0);
        area_pdf *= type_prob;
        sdir = pos - lp;
        lp_cos = dot(sdir, ln);
        if (lp_cos <= 0.0f) return rgb(0, 0, 0);
        light_point = offset_origin(lp, ln);
        sdir = pos - light_point;
        dist2 = dot(sdir, sdir);
        trace_length = std::sqrt(dist2);
        sdir = sdir * (1.0f / trace_length);
        lp_cos /= trace_length;
    }
    if (any_hit(S, light_point, sdir, trace_length * 0.9999f)) return rgb(0, 0, 0);
    float vis = 1.0f;
    float t0, t1;
    if (!s.volume_disabled && clip_ray(s.bbox_min, s.bbox_max, light_point, sdir, 0.0f, trace_length, &t0, &t1)) {
        float t = std::fmax(0.0f, t0);
        if (track(s, rng, light_point, sdir, &t, t1, true, &vis, shadow_steps, lookups) == SEG_CAP) {
            *capped = true;
            return rgb(0, 0, 0);
        }
    }
    if (!(vis > 0.0f)) return rgb(0, 0, 0);
    RGB fs;
    float bsdf_pdf, sp_cos;
    if (surf) {
        const V3 vin = to_local(surf->sf, -sdir);
        fs = brdf_eval(*f, q, vin);
        bsdf_pdf = brdf_pdf(*f, q, vin);
        sp_cos = std::fabs(dot(sdir, surf->gn));
    } else {
        const V3 vin = to_local(fr, -sdir);
        const float pf = phase_pdf(s.phase_kind, s.phase_param, vin);
        fs = rgb(s.albedo, s.albedo, s.albedo) * pf;
        bsdf_pdf = pf;
        sp_cos = 1.0f;
    }
    if (pick_sun) return fs * emittance * (surf ? vis * sp_cos / area_pdf : vis / area_pdf);
    float bp = bsdf_pdf * lp_cos / dist2;
    if (!std::isfinite(bp)) bp = 0.0f;
    const float mis = (area_pdf * area_pdf) / ((bp * bp) + (area_pdf * area_pdf));
    const RGB le = div(emittance, kPi);
    const float g = surf ? lp_cos * sp_cos / dist2 : lp_cos * 1.0f / dist2;
    return fs * le * (vis * mis * g / area_pdf);
}

// RadianceQuery of an in-medium vertex (optix_pathtracing_kernels.cu:14-29; the medium's
// surface parameters are common_renderer_types.h:2133-2140): position in the world box,
// normal = vOut (polar angles, slots in the reference's order), roughness 0 (or the local
// density / density_coeff when density queries are on), diffuse = albedo, specular = 0.
void write_query(const OrcScene& s, float* q, V3 pos, V3 vout, float roughness) {
    const float d[3] = {s.world_max[0] - s.world_min[0], s.world_max[1] - s.world_min[1],
                        s.world_max[2] - s.world_min[2]};
    const float r[3] = {pos.x - s.world_min[0], pos.y - s.world_min[1], pos.z - s.world_min[2]};
    for (int a = 0; a < 3; ++a) q[a] = d[a] != 0 ? r[a] / d[a] : 0.0f;
    float th, ph;
    to_polar_yup(vout, &th, &ph);
    q[3] = th;
    q[4] = ph;
    q[5] = th;
    q[6] = ph;
    q[7] = roughness;
    q[8] = q[9] = q[10] = s.albedo;
    q[11] = q[12] = q[13] = 0.0f;
}

// RadianceQuery of a surface vertex (optix_pathtracing_kernels.cu:14-29 with getSurfaceParameters,
// common_renderer_types.h:1491-1496 Lambert, 1671-1677 dichromatic): position in the world box,
// shading normal and vOut as polar angles, roughness, diffuse and specular reflectance.
void write_query_surf(const OrcScene& s, float* q, V3 pos, V3 normal, V3 vout, const OrcSurfaces::Mat& m) {
    const float d[3] = {s.world_max[0] - s.world_min[0], s.world_max[1] - s.world_min[1],
                        s.world_max[2] - s.world_min[2]};
    const float r[3] = {pos.x - s.world_min[0], pos.y - s.world_min[1], pos.z - s.world_min[2]};
    for (int a = 0; a < 3; ++a) q[a] = d[a] != 0 ? r[a] / d[a] : 0.0f;
    float th, ph;
    to_polar_yup(normal, &th, &ph);
    q[3] = th;
    q[4] = ph;
    to_polar_yup(vout, &th, &ph);
    q[5] = th;
    q[6] = ph;
    q[7] = m.roughness;
    for (int a = 0; a < 3; ++a) {
        q[8 + a] = m.diffuse[a];
        q[11 + a] = m.specular[a];
    }
}

inline uint32_t suffix_bits(uint32_t prev, uint32_t has_query, uint32_t path_length, uint32_t unbiased) {
    return (prev & ORC_NRC_INVALID_VERTEX) | ((has_query & 1u) << 22) | ((path_length & 0xFFu) << 23) |
           ((unbiased & 1u) << 31);
}

// optix_pathtracing_kernels.cu:31-434. nrc == nullptr: pathTrace (withNRC = false). Otherwise
// pathTraceWithNRC (mode 1) or generateTrainingData (mode 2) writing the pass's records for
// pixel `item` of the pass image.
RGB trace_path(const OrcScene& s, Pcg32& rng, int px, int py, uint32_t rec[4], int64_t* lookups,
               const OrcNrcSink* nrc = nullptr, uint32_t item = 0, bool unbiased = false) {
    const bool with_nrc = nrc != nullptr;
    const bool train = with_nrc && nrc->mode == 2;
    const float term_factor = with_nrc && nrc->termination > 0 ? nrc->termination : ORC_NRC_TERMINATION_FACTOR;
    const float train_term_factor = with_nrc && nrc->train_termination > 0 ? nrc->train_termination : 2 * term_factor;
    const float img_w = with_nrc ? static_cast<float>(nrc->img_w) : static_cast<float>(s.width);
    const float img_h = with_nrc ? static_cast<float>(nrc->img_h) : static_cast<float>(s.height);
    V3 origin, dir;
    float dir_pdf;
    {
        float ux = rng.uniform();
        float fx = (px + ux) / img_w;
        float uy = rng.uniform();
        float fy = (py + uy) / img_h;
        float vh = 2 * std::tan(s.cam_fovy * 0.5f);
        float vw = s.cam_aspect * vh;
        float sensor_area = vw * vh;
        origin = v3(s.cam_pos[0], s.cam_pos[1], s.cam_pos[2]);
        V3 local = normalize(v3(vw * (-0.5f + fx), vh * (0.5f - fy), -1));
        dir = normalize(mul(quat_to_m3(s.cam_quat), local));
        float az = std::fabs(local.z);
        dir_pdf = 1 / (az * az * az * sensor_area);
    }
    RGB contribution = rgb(0, 0, 0);
    float inv = 1.0f / dir_pdf;
    RGB throughput = rgb(1, 1, 1) * inv;
    const float init_importance = luminance(throughput);
    uint32_t path_length = 0;
    uint32_t end_code = 0;
    float primary_spread = 0.0f, sqrt_spread = 0.0f;
    uint32_t prev_vertex = ORC_NRC_INVALID_VERTEX;
    RGB prev_local_tp = rgb(0, 0, 0);
    bool terminal_written = false;
    while (true) {
        ++path_length;
        if (path_length > kHardVertexCap) {
            end_code = ORC_END_MAX_BOUNCES;
            break;
        }
        bool collided = false;
        float hit_dist = 1e10f;
        // optix_pathtracing_kernels.cu:84-96: the closest triangle bounds the segment.
        int32_t hit_tri = -1;
        float hb1 = 0.0f, hb2 = 0.0f;
        if (s.surfaces) {
            float th;
            hit_tri = closest_hit(*s.surfaces, origin, dir, 1e10f, &th, &hb1, &hb2);
            if (hit_tri >= 0) hit_dist = th;
        }
        float t0, t1;
        if (!s.volume_disabled && clip_ray(s.bbox_min, s.bbox_max, origin, dir, 0.0f, hit_dist, &t0, &t1)) {
            float t = std::fmax(0.0f, t0);
            float unused = 1.0f;
            SegEnd e = track(s, rng, origin, dir, &t, t1, false, &unused, &rec[1], lookups);
            if (e == SEG_CAP) {
                end_code = ORC_END_STEP_CAP;
                break;
            }
            if (e == SEG_COLLIDE) {
                collided = true;
                hit_dist = t;
            }
        }
        if (!collided && hit_tri >= 0) {
            // A triangle hit: surface point, path spread, emission against area-light sampling
            // (:176-239), Russian roulette and the radiance-cache end (:254-330), NEE, BSDF
            // sampling, the offset origin and the training vertex (:332-409).
            const OrcSurfaces& S = *s.surfaces;
            const SurfPt sp = surface_point(S, static_cast<uint32_t>(hit_tri), hb1, hb2, s.env_enabled != 0);
            const V3 ray_origin = origin;
            const V3 q = to_local(sp.sf, -dir);
            const OrcSurfaces::Mat& mt = S.mats[sp.material];
            if (with_nrc) {
                // :200-210, |cos| against the geometric normal.
                const V3 dv = ray_origin - sp.pos;
                const float dist2 = dv.x * dv.x + dv.y * dv.y + dv.z * dv.z;
                const float abs_dot = std::fabs(dot(dir, sp.gn));
                if (path_length == 1)
                    primary_spread = dist2 / (4 * kPi * abs_dot);
                else
                    sqrt_spread += std::sqrt(dist2 / (dir_pdf * abs_dot));
            }
            if (q.z > 0 && mt.emissive) {
                float mis = 1.0f;
                if (path_length > 1) {
                    const V3 dv = ray_origin - sp.pos;
                    const float dist2 = dot(dv, dv);
                    const float light_pdf = sp.hyp_area_pdf * dist2 / q.z;
                    const float bsdf_pdf = dir_pdf;
                    mis = (bsdf_pdf * bsdf_pdf) / ((bsdf_pdf * bsdf_pdf) + (light_pdf * light_pdf));
                }
                const RGB implicit = rgb(mt.emit[0], mt.emit[1], mt.emit[2]) * (mis / kPi);
                if (!train) contribution = contribution + throughput * implicit;
                if (train && prev_vertex != ORC_NRC_INVALID_VERTEX) {
                    float* tg = nrc->train_target + 3 * static_cast<size_t>(prev_vertex);
                    const RGB add = prev_local_tp * implicit;
                    tg[0] += add.r;
                    tg[1] += add.g;
                    tg[2] += add.b;
                }
            }
            float continue_prob = 1.0f;
            bool rr_kill = false;
            const int32_t rr_from = train ? std::max(s.rr_start, 3) : s.rr_start;
            if (static_cast<int32_t>(path_length) >= rr_from) {
                continue_prob = std::fmin(luminance(throughput) / init_importance, 1.0f);
                if (rng.uniform() >= continue_prob) rr_kill = true;
            }
            if (!with_nrc && rr_kill) {
                end_code = ORC_END_RR;
                break;
            }
            if (with_nrc) {
                bool ends_with_cache = rr_kill;
                const float spread2 = sqrt_spread * sqrt_spread;
                if (train) {
                    if (!unbiased) ends_with_cache |= spread2 > train_term_factor * primary_spread;
                } else {
                    ends_with_cache |= spread2 > term_factor * primary_spread;
                }
                if (ends_with_cache) {
                    write_query_surf(s, nrc->infer_query + ORC_NRC_QUERY_FLOATS * static_cast<size_t>(item), sp.pos,
                                     sp.sf.n, -dir, mt);
                    if (train) {
                        nrc->train_suffix[item] = suffix_bits(prev_vertex, 1, path_length, unbiased ? 1 : 0);
                    } else {
                        float* tp = nrc->terminal_tp + 3 * static_cast<size_t>(item);
                        tp[0] = throughput.r;
                        tp[1] = throughput.g;
                        tp[2] = throughput.b;
                        nrc->terminal_bits[item] = 1u | ((path_length & 0xFFu) << 1);
                    }
                    terminal_written = true;
                    end_code = ORC_END_CACHE;
                    break;
                }
            }
            throughput = div(throughput, continue_prob);
            const Brdf f = brdf_of(mt);
            bool capped = false;
            OrcScene s_nee = s;
            if (train) s_nee.shadow_rr = 0.0f;
            const RGB nee = next_event_surf(s_nee, rng, sp.pos, sp.sf, &sp, &f, q, &rec[2], lookups, &capped);
            if (capped) {
                end_code = ORC_END_STEP_CAP;
                break;
            }
            if (!train) contribution = contribution + throughput * nee;
            if (s.max_bounces > 0 && static_cast<int32_t>(path_length) >= s.max_bounces) {
                end_code = ORC_END_MAX_BOUNCES;
                break;
            }
            const float u0 = rng.uniform();
            const float u1 = rng.uniform();
            V3 local;
            float pdf;
            const RGB fs = brdf_sample(f, q, u0, u1, &local, &pdf);
            if (pdf == 0.0f) {
                end_code = ORC_END_PDF_ZERO;
                break;
            }
            const V3 v_out = -dir;
            dir = from_local(sp.sf, local);
            const float dot_sgn = dot(dir, sp.gn);
            const RGB local_tp = fs * (std::fabs(dot_sgn) / pdf);
            throughput = throughput * local_tp;
            origin = offset_origin(sp.pos, (dot_sgn > 0.0f ? 1.0f : -1.0f) * sp.gn);
            dir_pdf = pdf;
            if (train) {
                const uint32_t idx = (*nrc->num_train)++;
                if (idx < ORC_NRC_TRAIN_BUFFER_SIZE) {
                    write_query_surf(s, nrc->train_query + ORC_NRC_QUERY_FLOATS * static_cast<size_t>(idx), sp.pos,
                                     sp.sf.n, v_out, mt);
                    float* lt = nrc->train_local_tp + 3 * static_cast<size_t>(idx);
                    lt[0] = local_tp.r;
                    lt[1] = local_tp.g;
                    lt[2] = local_tp.b;
                    nrc->train_bits[idx] = (prev_vertex & ORC_NRC_INVALID_VERTEX) | ((path_length & 0xFFu) << 22) |
                                           ((unbiased ? 1u : 0u) << 30);
                    float* tg = nrc->train_target + 3 * static_cast<size_t>(idx);
                    tg[0] = nee.r;
                    tg[1] = nee.g;
                    tg[2] = nee.b;
                    prev_local_tp = local_tp;
                    prev_vertex = idx;
                } else {
                    write_query_surf(s, nrc->infer_query + ORC_NRC_QUERY_FLOATS * static_cast<size_t>(item), sp.pos,
                                     sp.sf.n, v_out, mt);
                    nrc->train_suffix[item] = suffix_bits(prev_vertex, 1, path_length, unbiased ? 1 : 0);
                    terminal_written = true;
                    end_code = ORC_END_TRAIN_FULL;
                    break;
                }
            }
            continue;
        }
        if (!collided) {
            // optix_pathtracing_kernels.cu:130-174 (environment hit with MIS).
            if (s.env_enabled) {
                float hyp_pdf;
                RGB radiance = env_evaluate(s, dir, &hyp_pdf);
                float mis = 1.0f;
                if (path_length > 1) {
                    float sel = s.sun_enabled ? (1.0f - s.sun_prob) : 1.0f;
                    // :140-142: with emitting triangles the environment is picked with probToSampleEnvLight.
                    if (s.surfaces && s.surfaces->inst_integral > 0.0f) sel = s.sun_enabled ? 0.25f * sel : 0.25f;
                    float light_pdf = sel * hyp_pdf;
                    float bsdf_pdf = dir_pdf;
                    mis = (bsdf_pdf * bsdf_pdf) / ((bsdf_pdf * bsdf_pdf) + (light_pdf * light_pdf));
                }
                RGB implicit = radiance * mis;
                if (!train) contribution = contribution + throughput * implicit;
                if (train && prev_vertex != ORC_NRC_INVALID_VERTEX) {
                    float* tg = nrc->train_target + 3 * static_cast<size_t>(prev_vertex);
                    RGB add = prev_local_tp * implicit;
                    tg[0] += add.r;
                    tg[1] += add.g;
                    tg[2] += add.b;
                }
            }
            end_code = ORC_END_ESCAPE;
            break;
        }
        const V3 seg_origin = origin;
        V3 pos = origin + hit_dist * dir;
        Frame fr = make_frame(-dir);
        if (with_nrc) {
            // :200-210, |cos| = 1 in a medium.
            V3 dv = seg_origin - pos;
            float dist2 = dv.x * dv.x + dv.y * dv.y + dv.z * dv.z;
            if (path_length == 1)
                primary_spread = dist2 / (4 * kPi * 1.0f);
            else
                sqrt_spread += std::sqrt(dist2 / (dir_pdf * 1.0f));
        }

        // Russian roulette (:254-268), from the third vertex in the training pass.
        float continue_prob = 1.0f;
        bool rr_kill = false;
        const int32_t rr_from = train ? std::max(s.rr_start, 3) : s.rr_start;
        if (static_cast<int32_t>(path_length) >= rr_from) {
            continue_prob = std::fmin(luminance(throughput) / init_importance, 1.0f);
            if (rng.uniform() >= continue_prob) rr_kill = true;
        }
        if (!with_nrc && rr_kill) {
            end_code = ORC_END_RR;
            break;
        }
        if (with_nrc) {
            // :282-330: end with a cache query on RR or when the spread is large enough.
            bool ends_with_cache = rr_kill;
            const float spread2 = sqrt_spread * sqrt_spread;
            if (train) {
                if (!unbiased) ends_with_cache |= spread2 > train_term_factor * primary_spread;
            } else {
                ends_with_cache |= spread2 > term_factor * primary_spread;
            }
            if (ends_with_cache) {
                float rough = 0.0f;
                if (nrc->density_query && s.density_coeff > 0) rough = density_at(s, seg_origin, dir, hit_dist) / s.density_coeff;
                write_query(s, nrc->infer_query + ORC_NRC_QUERY_FLOATS * static_cast<size_t>(item), pos, -dir, rough);
                if (train) {
                    nrc->train_suffix[item] = suffix_bits(prev_vertex, 1, path_length, unbiased ? 1 : 0);
                } else {
                    float* tp = nrc->terminal_tp + 3 * static_cast<size_t>(item);
                    tp[0] = throughput.r;
                    tp[1] = throughput.g;
                    tp[2] = throughput.b;
                    nrc->terminal_bits[item] = 1u | ((path_length & 0xFFu) << 1);
                }
                terminal_written = true;
                end_code = ORC_END_CACHE;
                break;
            }
        }
        throughput = div(throughput, continue_prob);

        float vis;
        bool capped = false;
        // Training suffixes keep plain ratio tracking (no roulette): their NEE estimates are the
        // cache's targets.
        OrcScene s_nee = s;
        if (train) s_nee.shadow_rr = 0.0f;
        RGB nee = s.surfaces ? next_event_surf(s_nee, rng, pos, fr, nullptr, nullptr, v3(0, 0, 1), &rec[2], lookups, &capped)
                             : next_event(s_nee, rng, pos, fr, &vis, &rec[2], lookups, &capped);
        if (capped) {
            end_code = ORC_END_STEP_CAP;
            break;
        }
        if (!train) contribution = contribution + throughput * nee;

        if (s.max_bounces > 0 && static_cast<int32_t>(path_length) >= s.max_bounces) {
            end_code = ORC_END_MAX_BOUNCES;
            break;
        }
        float u0 = rng.uniform();
        float u1 = rng.uniform();
        V3 local;
        float pdf = phase_sample(s.phase_kind, s.phase_param, u0, u1, &local);
        if (pdf == 0.0f) {
            end_code = ORC_END_PDF_ZERO;
            break;
        }
        RGB fs = rgb(s.albedo, s.albedo, s.albedo) * pdf;
        const V3 v_out = -dir;
        dir = from_local(fr, local);
        RGB local_tp = fs * (std::fabs(1.0f) / pdf);
        throughput = throughput * local_tp;
        origin = pos;
        dir_pdf = pdf;
        if (train) {
            // :358-409: training vertex (vertices numbered in the order they are made).
            const uint32_t idx = (*nrc->num_train)++;
            float rough = 0.0f;
            if (nrc->density_query && s.density_coeff > 0) rough = density_at(s, seg_origin, v_out * -1.0f, hit_dist) / s.density_coeff;
            if (idx < ORC_NRC_TRAIN_BUFFER_SIZE) {
                write_query(s, nrc->train_query + ORC_NRC_QUERY_FLOATS * static_cast<size_t>(idx), pos, v_out, rough);
                float* lt = nrc->train_local_tp + 3 * static_cast<size_t>(idx);
                lt[0] = local_tp.r;
                lt[1] = local_tp.g;
                lt[2] = local_tp.b;
                nrc->train_bits[idx] = (prev_vertex & ORC_NRC_INVALID_VERTEX) | ((path_length & 0xFFu) << 22) |
                                       ((unbiased ? 1u : 0u) << 30);
                float* tg = nrc->train_target + 3 * static_cast<size_t>(idx);
                tg[0] = nee.r;
                tg[1] = nee.g;
                tg[2] = nee.b;
                prev_local_tp = local_tp;
                prev_vertex = idx;
            } else {
                write_query(s, nrc->infer_query + ORC_NRC_QUERY_FLOATS * static_cast<size_t>(item), pos, v_out, rough);
                nrc->train_suffix[item] = suffix_bits(prev_vertex, 1, path_length, unbiased ? 1 : 0);
                terminal_written = true;
                end_code = ORC_END_TRAIN_FULL;
                break;
            }
        }
    }
    if (with_nrc && !terminal_written) {
        if (train) {
            nrc->train_suffix[item] = suffix_bits(prev_vertex, 0, path_length, unbiased ? 1 : 0);
        } else {
            float* tp = nrc->terminal_tp + 3 * static_cast<size_t>(item);
            tp[0] = throughput.r;
            tp[1] = throughput.g;
            tp[2] = throughput.b;
            nrc->terminal_bits[item] = (path_length & 0xFFu) << 1;
        }
    }
    rec[0] = path_length;
    rec[3] = end_code;
    return contribution;
}

}  // namespace

extern "C" {

int orc_version(void) { return 1; }

// renderer_main.cpp:86-93: one std::mt19937_64 stream, row-major pixel order.
void orc_seed_states(int32_t width, int32_t height, uint64_t seed, uint64_t* out) {
    std::mt19937_64 gen(seed);
    for (int64_t i = 0; i < static_cast<int64_t>(width) * height; ++i) out[i] = gen();
}

void orc_pcg_floats(uint64_t state, int32_t n, float* out, uint64_t* state_out) {
    Pcg32 r{state};
    for (int i = 0; i < n; ++i) out[i] = r.uniform();
    if (state_out) *state_out = r.state;
}

// renderer_scene.h:1185-1198: map dims are next powers of two with height >= width / 2.
int64_t orc_imp_map_size(int32_t env_w, int32_t env_h, int32_t* map_w, int32_t* map_h, int32_t* num_mips,
                         int64_t* offsets) {
    auto next_pow2 = [](uint32_t v) {
        uint32_t p = 1;
        while (p < v) p <<= 1;
        return p;
    };
    uint32_t dx = next_pow2(env_w);
    uint32_t dy = std::max(next_pow2(env_h), dx >> 1);
    int levels = 1;
    while ((1u << (levels - 1)) < dx) ++levels;
    *map_w = dx;
    *map_h = dy;
    *num_mips = levels;
    int64_t off = 0;
    for (int l = 0; l < levels; ++l) {
        if (offsets) offsets[l] = off;
        int64_t w = std::max<int64_t>(dx >> l, 1), h = std::max<int64_t>(dy >> l, 1);
        off += w * h;
    }
    return off;
}

// compute_light_probs.cu:161-211. Returns the integral written by the last level.
float orc_build_imp_map(const float* env_rgb, int32_t env_w, int32_t env_h, float* mips) {
    int32_t mw, mh, nm;
    int64_t offs[32];
    orc_imp_map_size(env_w, env_h, &mw, &mh, &nm, offs);
    for (int y = 0; y < mh; ++y) {
        for (int x = 0; x < mw; ++x) {
            float importance = 0.0f;
            if (x < env_w && y < env_h) {
                const float* p = env_rgb + 3 * (static_cast<int64_t>(y) * env_w + x);
                RGB c = rgb(p[0], p[1], p[2]);
                float correction = kPi / 2 * std::sin(kPi * (y + 0.5f) / env_h);
                importance = luminance(c) * correction;
            }
            mips[offs[0] + static_cast<int64_t>(y) * mw + x] = importance;
        }
    }
    float integral = 0.0f;
    for (int l = 1; l < nm; ++l) {
        int sw = mw >> (l - 1), sh = mh >> (l - 1);
        int dw = std::max(mw >> l, 1), dh = std::max(mh >> l, 1);
        for (int y = 0; y < dh; ++y) {
            for (int x = 0; x < dw; ++x) {
                float sum = 0.0f;
                int xs[4] = {2 * x, 2 * x + 1, 2 * x, 2 * x + 1};
                int ys[4] = {2 * y, 2 * y, 2 * y + 1, 2 * y + 1};
                for (int q = 0; q < 4; ++q) {
                    if (xs[q] < sw && ys[q] < sh)
                        sum += mips[offs[l - 1] + static_cast<int64_t>(ys[q]) * std::max(sw, 1) + xs[q]];
                }
                sum *= 0.25f;
                mips[offs[l] + static_cast<int64_t>(y) * dw + x] = sum;
                if (l == nm - 1) integral = sum * static_cast<float>(1u << (2 * (nm - 1)));
            }
        }
    }
    return integral;
}

// Majorant cells of the config mode: max over voxels [8c-1, 8c+9] of each 8^3 cell and the
// reference's global majorant over index coordinates [0, n-1) (renderer_scene.cpp:498-509).
float orc_majorants(const float* v, int32_t nx, int32_t ny, int32_t nz, float* cells) {
    int lx = (nx + 7) / 8, ly = (ny + 7) / 8, lz = (nz + 7) / 8;
    auto at = [&](int x, int y, int z) -> float {
        if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return 0.0f;
        return v[(static_cast<int64_t>(x) * ny + y) * nz + z];
    };
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int cx = 0; cx < lx; ++cx)
        for (int cy = 0; cy < ly; ++cy)
            for (int cz = 0; cz < lz; ++cz) {
                float m = 0.0f;
                for (int x = 8 * cx - 1; x <= 8 * cx + 9; ++x)
                    for (int y = 8 * cy - 1; y <= 8 * cy + 9; ++y)
                        for (int z = 8 * cz - 1; z <= 8 * cz + 9; ++z) m = std::max(m, at(x, y, z));
                cells[(static_cast<int64_t>(cx) * ly + cy) * lz + cz] = m;
            }
    float g = -INFINITY;
    for (int x = 0; x < nx - 1; ++x)
        for (int y = 0; y < ny - 1; ++y)
            for (int z = 0; z < nz - 1; ++z) g = std::max(g, at(x, y, z));
    return g;
}

// sRGB_gamma_s (basic_types.h:3181-3188).
void orc_srgb_gamma(const float* in, int32_t n, float* out) {
    for (int32_t i = 0; i < n; ++i) {
        const float v = in[i];
        out[i] = v <= 0.0031308f ? 12.92f * v : 1.055f * std::pow(v, static_cast<float>(1 / 2.4)) - 0.055f;
    }
}

// applyToneMap (renderer/gpu_kernels/post_process_kernels.cu:10-41) and the 8-bit conversion of
// saveImage (common/common_host.cpp:517-568) with the headless loop's settings
// (renderer_main.cpp:1490-1495): x^(1/0.6) per channel, colour * (1 - exp(-b * lum)) / lum,
// negatives clamped to 0, sRGB_gamma_s (basic_types.h:3181-3188) when srgb is set,
// min(uint(v * 255), 255) per channel (NaN -> 0), alpha 255.
void orc_tonemap(const float* mean, int32_t n, float brightness, int32_t srgb, float* out_rgb, uint8_t* out_rgba) {
    auto gamma_s = [](float v) {
        if (v <= 0.0031308f) return 12.92f * v;
        return 1.055f * std::pow(v, static_cast<float>(1 / 2.4)) - 0.055f;
    };
    auto to_byte = [](float v) -> uint8_t {
        const float x = v * 255.0f;
        if (!(x > 0.0f)) return 0;
        if (x >= 255.0f) return 255;
        return static_cast<uint8_t>(static_cast<uint32_t>(x));
    };
    for (int32_t i = 0; i < n; ++i) {
        constexpr float kGamma = 1.0f / 0.6f;
        float c[3] = {std::pow(mean[3 * i], kGamma), std::pow(mean[3 * i + 1], kGamma),
                      std::pow(mean[3 * i + 2], kGamma)};
        const float lum = 0.2126729f * c[0] + 0.7151522f * c[1] + 0.0721750f * c[2];
        if (lum > 0.0f) {
            const float lum_t = 1 - std::exp(-brightness * lum);
            const float sc = lum_t / lum;
            for (float& v : c) v *= sc;
        }
        for (int k = 0; k < 3; ++k) {
            if (out_rgb) out_rgb[3 * i + k] = c[k];
            float v = std::fmax(c[k], 0.0f);
            if (srgb) v = gamma_s(v);
            if (out_rgba) out_rgba[4 * i + k] = to_byte(v);
        }
        if (out_rgba) out_rgba[4 * i + 3] = 255;
    }
}

void orc_sample_density(const OrcScene* sc, const float* idx, int32_t n, float* out) {
    for (int i = 0; i < n; ++i) out[i] = sample_trilinear(*sc, v3(idx[3 * i], idx[3 * i + 1], idx[3 * i + 2]));
}

void orc_clip_rays(const OrcScene* sc, const float* org, const float* dir, int32_t n, float* t0, float* t1,
                   int32_t* hit) {
    for (int i = 0; i < n; ++i) {
        float a = 0, b = 0;
        hit[i] = clip_ray(sc->bbox_min, sc->bbox_max, v3(org[3 * i], org[3 * i + 1], org[3 * i + 2]),
                          v3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]), 0.0f, 1e10f, &a, &b);
        t0[i] = a;
        t1[i] = b;
    }
}

void orc_env_sample(const OrcScene* sc, const float* u, int32_t n, float* dir, float* pdf, float* out) {
    for (int i = 0; i < n; ++i) {
        V3 d;
        float p;
        RGB c = env_sample(*sc, u[2 * i], u[2 * i + 1], &d, &p);
        dir[3 * i] = d.x;
        dir[3 * i + 1] = d.y;
        dir[3 * i + 2] = d.z;
        pdf[i] = p;
        out[3 * i] = c.r;
        out[3 * i + 1] = c.g;
        out[3 * i + 2] = c.b;
    }
}

// The hierarchical importance walk alone: per u pair, (pixel x, pixel y, remapped u0, u1, prob).
void orc_imp_sample(const OrcScene* sc, const float* u, int32_t n, float* out) {
    for (int i = 0; i < n; ++i) {
        int px, py;
        float r0, r1, prob;
        imp_sample(*sc, u[2 * i], u[2 * i + 1], &px, &py, &r0, &r1, &prob);
        out[5 * i] = static_cast<float>(px);
        out[5 * i + 1] = static_cast<float>(py);
        out[5 * i + 2] = r0;
        out[5 * i + 3] = r1;
        out[5 * i + 4] = prob;
    }
}

void orc_env_evaluate(const OrcScene* sc, const float* dir, int32_t n, float* pdf, float* out) {
    for (int i = 0; i < n; ++i) {
        float p;
        RGB c = env_evaluate(*sc, v3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]), &p);
        pdf[i] = p;
        out[3 * i] = c.r;
        out[3 * i + 1] = c.g;
        out[3 * i + 2] = c.b;
    }
}

void orc_phase_sample(int32_t kind, float param, const float* u, int32_t n, float* dl, float* pdf) {
    for (int i = 0; i < n; ++i) {
        V3 l;
        pdf[i] = phase_sample(kind, param, u[2 * i], u[2 * i + 1], &l);
        dl[3 * i] = l.x;
        dl[3 * i + 1] = l.y;
        dl[3 * i + 2] = l.z;
    }
}

void orc_phase_eval(int32_t kind, float param, const float* dl, int32_t n, float* pdf) {
    for (int i = 0; i < n; ++i) pdf[i] = phase_pdf(kind, param, v3(dl[3 * i], dl[3 * i + 1], dl[3 * i + 2]));
}

void orc_polar_yup(const float* v, int32_t n, float* tp) {
    for (int i = 0; i < n; ++i) to_polar_yup(v3(v[3 * i], v[3 * i + 1], v[3 * i + 2]), &tp[2 * i], &tp[2 * i + 1]);
}

void orc_coordinate_system(const float* nrm, int32_t n, float* tb) {
    for (int i = 0; i < n; ++i) {
        Frame f = make_frame(v3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]));
        float vals[6] = {f.t.x, f.t.y, f.t.z, f.b.x, f.b.y, f.b.z};
        std::memcpy(tb + 6 * i, vals, sizeof(vals));
    }
}

void orc_quat_to_matrix(const float* q, float* m9) {
    M3 m = quat_to_m3(q);
    float vals[9] = {m.c0.x, m.c0.y, m.c0.z, m.c1.x, m.c1.y, m.c1.z, m.c2.x, m.c2.y, m.c2.z};
    std::memcpy(m9, vals, sizeof(vals));
}

OrcSurfaces* orc_surfaces_create(const OrcSurfMaterial* mats, uint32_t nmat, const OrcSurfGeometry* geoms, uint32_t ngeom,
                                 const OrcSurfInstance* insts, uint32_t ninst, float* box_out) {
    if (!mats || !geoms || !insts || nmat == 0 || ngeom == 0 || ninst == 0) return nullptr;
    auto* S = new OrcSurfaces();
    for (uint32_t k = 0; k < nmat; ++k) {
        const OrcSurfaces::Mat d = decode_material(mats[k]);
        S->mats.push_back(d);
    }
    std::vector<float> glo(3 * static_cast<size_t>(ngeom), INFINITY), ghi(3 * static_cast<size_t>(ngeom), -INFINITY);
    for (uint32_t g = 0; g < ngeom; ++g) {
        const OrcSurfGeometry& G = geoms[g];
        if (G.material >= nmat) {
            delete S;
            return nullptr;
        }
        OrcSurfaces::Geom d;
        d.num_tris = G.num_triangles;
        d.material = G.material;
        for (uint32_t v = 0; v < G.num_vertices; ++v) {
            const float* a = G.vertices + 9 * static_cast<size_t>(v);
            for (int k = 0; k < 3; ++k) {
                glo[3 * g + k] = std::min(glo[3 * g + k], a[k]);
                ghi[3 * g + k] = std::max(ghi[3 * g + k], a[k]);
                d.nrm.push_back(a[3 + k]);
                d.tan.push_back(a[6 + k]);
            }
        }
        const OrcSurfaces::Mat& mt = S->mats[G.material];
        for (uint32_t t = 0; t < G.num_triangles; ++t) {
            const uint32_t* ix = G.triangles + 3 * static_cast<size_t>(t);
            d.tri.insert(d.tri.end(), ix, ix + 3);
            // computeTriangleImportance (compute_light_probs.cu:19-50), object-space area.
            const float* p0 = G.vertices + 9 * static_cast<size_t>(ix[0]);
            const float* p1 = G.vertices + 9 * static_cast<size_t>(ix[1]);
            const float* p2 = G.vertices + 9 * static_cast<size_t>(ix[2]);
            const V3 n = cross3(v3(p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]), v3(p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]));
            const float area = 0.5f * std::sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
            RGB est = rgb(0, 0, 0);
            if (mt.emissive) {
                const RGB e = rgb(mt.emit[0], mt.emit[1], mt.emit[2]);
                est = est + e;
                est = est + e;
                est = est + e;
                est = est * (1.0f / 3);
            }
            d.w.push_back(luminance(est) * area);
        }
        d.integral = excl_cdf(d.w, &d.cdf);
        S->geoms.push_back(std::move(d));
    }
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < ninst; ++i) {
        const OrcSurfInstance& I = insts[i];
        if (I.num_geometries == 0 || static_cast<uint64_t>(I.first_geometry) + I.num_geometries > ngeom) {
            delete S;
            return nullptr;
        }
        OrcSurfaces::Inst d;
        std::memcpy(d.m, I.transform, sizeof(d.m));
        // Normals go through the inverse transpose (common_renderer_types.h:1080-1085), the
        // inverse taken in double.
        const double a = I.transform[0], b = I.transform[1], c = I.transform[2], dd = I.transform[4],
                     e = I.transform[5], f = I.transform[6], g = I.transform[8], h = I.transform[9],
                     k = I.transform[10];
        const double A = e * k - f * h, B = -(dd * k - f * g), Cc = dd * h - e * g;
        const double r = 1.0 / (a * A + b * B + c * Cc);
        const double inv[9] = {A * r, -(b * k - c * h) * r, (b * f - c * e) * r, B * r, (a * k - c * g) * r,
                               -(a * f - c * dd) * r, Cc * r, -(a * h - b * g) * r, (a * e - b * dd) * r};
        for (int row = 0; row < 3; ++row)
            for (int col = 0; col < 3; ++col) d.nm[3 * row + col] = static_cast<float>(inv[3 * col + row]);
        d.uniform_scale = I.uniform_scale;
        d.first_geom = I.first_geometry;
        d.num_geoms = I.num_geometries;
        d.first_world_tri_of_geom0 = static_cast<uint32_t>(S->inst_geom_first_tri.size());
        for (uint32_t q = 0; q < I.num_geometries; ++q) d.group_w.push_back(S->geoms[I.first_geometry + q].integral);
        d.group_integral = excl_cdf(d.group_w, &d.group_cdf);
        const float* M = I.transform;
        const float col0 = std::sqrt(M[0] * M[0] + M[4] * M[4] + M[8] * M[8]);
        S->inst_w.push_back((col0 * col0) * d.group_integral);
        // World box: the group's object box transformed corner by corner (basic_types.h:2876-2888).
        float gl[3] = {INFINITY, INFINITY, INFINITY}, gh[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t q = 0; q < I.num_geometries; ++q)
            for (int ax = 0; ax < 3; ++ax) {
                gl[ax] = std::min(gl[ax], glo[3 * (I.first_geometry + q) + ax]);
                gh[ax] = std::max(gh[ax], ghi[3 * (I.first_geometry + q) + ax]);
            }
        for (int corner = 0; corner < 8; ++corner) {
            const float pc[3] = {(corner & 1) ? gh[0] : gl[0], (corner & 2) ? gh[1] : gl[1], (corner & 4) ? gh[2] : gl[2]};
            const V3 w = xf_point(M, pc);
            const float wa[3] = {w.x, w.y, w.z};
            for (int ax = 0; ax < 3; ++ax) {
                lo[ax] = std::min(lo[ax], wa[ax]);
                hi[ax] = std::max(hi[ax], wa[ax]);
            }
        }
        for (uint32_t q = 0; q < I.num_geometries; ++q) {
            const uint32_t gidx = I.first_geometry + q;
            const OrcSurfGeometry& G = geoms[gidx];
            S->inst_geom_first_tri.push_back(static_cast<uint32_t>(S->owner_inst.size()));
            for (uint32_t t = 0; t < G.num_triangles; ++t) {
                for (int v = 0; v < 3; ++v) {
                    const V3 w = xf_point(M, G.vertices + 9 * static_cast<size_t>(G.triangles[3 * static_cast<size_t>(t) + v]));
                    S->pos.push_back(w.x);
                    S->pos.push_back(w.y);
                    S->pos.push_back(w.z);
                }
                S->owner_inst.push_back(i);
                S->owner_geom.push_back(gidx);
                S->owner_prim.push_back(t);
            }
        }
        S->insts.push_back(std::move(d));
    }
    S->inst_integral = excl_cdf(S->inst_w, &S->inst_cdf);
    if (box_out)
        for (int ax = 0; ax < 3; ++ax) {
            box_out[ax] = lo[ax];
            box_out[3 + ax] = hi[ax];
        }
    return S;
}

void orc_surfaces_destroy(OrcSurfaces* s) { delete s; }

void orc_surface_closest(const OrcSurfaces* S, const float* org, const float* dir, int32_t n, float tmax, int32_t* tri,
                         float* tb) {
    for (int32_t i = 0; i < n; ++i) {
        float t = 0, b1 = 0, b2 = 0;
        tri[i] = closest_hit(*S, v3(org[3 * i], org[3 * i + 1], org[3 * i + 2]), v3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]),
                             tmax, &t, &b1, &b2);
        tb[3 * i] = t;
        tb[3 * i + 1] = b1;
        tb[3 * i + 2] = b2;
    }
}

void orc_surface_any(const OrcSurfaces* S, const float* org, const float* dir, const float* tmax, int32_t n, int32_t* hit) {
    for (int32_t i = 0; i < n; ++i)
        hit[i] = any_hit(*S, v3(org[3 * i], org[3 * i + 1], org[3 * i + 2]), v3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]),
                         tmax[i]) ? 1 : 0;
}

void orc_offset_origin(const float* pn, int32_t n, float* out) {
    for (int32_t i = 0; i < n; ++i) {
        const V3 r = offset_origin(v3(pn[6 * i], pn[6 * i + 1], pn[6 * i + 2]), v3(pn[6 * i + 3], pn[6 * i + 4], pn[6 * i + 5]));
        out[3 * i] = r.x;
        out[3 * i + 1] = r.y;
        out[3 * i + 2] = r.z;
    }
}

static Brdf decoded_brdf(const OrcSurfMaterial* m) { return brdf_of(decode_material(*m)); }

void orc_bsdf_eval(const OrcSurfMaterial* m, const float* q, const float* v, int32_t n, float* val, float* pdf) {
    const Brdf f = decoded_brdf(m);
    for (int32_t i = 0; i < n; ++i) {
        const V3 qq = v3(q[3 * i], q[3 * i + 1], q[3 * i + 2]), vv = v3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        const RGB c = brdf_eval(f, qq, vv);
        val[3 * i] = c.r;
        val[3 * i + 1] = c.g;
        val[3 * i + 2] = c.b;
        pdf[i] = brdf_pdf(f, qq, vv);
    }
}

void orc_bsdf_sample(const OrcSurfMaterial* m, const float* q, const float* u, int32_t n, float* out7) {
    const Brdf f = decoded_brdf(m);
    for (int32_t i = 0; i < n; ++i) {
        V3 d;
        float pdf;
        const RGB c = brdf_sample(f, v3(q[3 * i], q[3 * i + 1], q[3 * i + 2]), u[2 * i], u[2 * i + 1], &d, &pdf);
        const float o[7] = {d.x, d.y, d.z, c.r, c.g, c.b, pdf};
        std::memcpy(out7 + 7 * i, o, sizeof(o));
    }
}

int64_t orc_render_plain(const OrcScene* sc, uint64_t* rng_states, int32_t accum_base, int32_t spp,
                         double* sum_rgb, float* mean_rgb, uint32_t* dlog, int32_t row0, int32_t row1,
                         int32_t nthreads) {
    const OrcScene& s = *sc;
    int64_t total = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
#endif
    for (int y = row0; y < row1; ++y) {
        for (int x = 0; x < s.width; ++x) {
            int64_t pix = static_cast<int64_t>(y) * s.width + x;
            Pcg32 rng{rng_states[pix]};
            for (int i = 0; i < spp; ++i) {
                if (s.stream_mode == 1)
                    rng.state = pcg_advance(rng_states[pix], static_cast<uint64_t>(accum_base + i) << kSampleStreamShift);
                uint32_t rec[4] = {0, 0, 0, 0};
                int64_t lk = 0;
                RGB c = trace_path(s, rng, x, y, rec, &lk);
                total += lk;
                if (dlog) std::memcpy(dlog + 4 * (pix * spp + i), rec, sizeof(rec));
                // optix_pathtracing_kernels.cu:415-432: drop non-finite / negative samples.
                if (!all_nonneg_finite(c)) continue;
                if (sum_rgb) {
                    sum_rgb[3 * pix] += c.r;
                    sum_rgb[3 * pix + 1] += c.g;
                    sum_rgb[3 * pix + 2] += c.b;
                }
                if (mean_rgb && s.stream_mode == 0) {
                    uint32_t n = static_cast<uint32_t>(accum_base + i);
                    RGB prev = rgb(0, 0, 0);
                    if (n > 0) prev = rgb(mean_rgb[3 * pix], mean_rgb[3 * pix + 1], mean_rgb[3 * pix + 2]);
                    float w = 1.0f / (n + 1);
                    RGB r = (1 - w) * prev + w * c;
                    mean_rgb[3 * pix] = r.r;
                    mean_rgb[3 * pix + 1] = r.g;
                    mean_rgb[3 * pix + 2] = r.b;
                }
            }
            if (s.stream_mode == 0) rng_states[pix] = rng.state;
        }
    }
    return total;
}

// One radiance-cache pass over the pass image (nrc->img_w x nrc->img_h pixels), pixels in
// row-major order, RNG states of the full image's per-pixel buffer.
int64_t orc_nrc_pass(const OrcScene* sc, uint64_t* rng_states, const OrcNrcSink* nrc, uint32_t* dlog) {
    const OrcScene& s = *sc;
    int64_t total = 0;
    for (uint32_t py = 0; py < nrc->img_h; ++py) {
        for (uint32_t px = 0; px < nrc->img_w; ++px) {
            const uint32_t item = py * nrc->img_w + px;
            const int64_t pix = static_cast<int64_t>(py) * s.width + px;
            Pcg32 rng{rng_states[pix]};
            // :60-66: one unbiased training suffix per 4x4 tile.
            const uint32_t tile = (py % 4) * 4 + (px % 4);
            const bool unbiased = nrc->mode == 2 && (tile + nrc->unbiased_offset) % 16 == 0;
            uint32_t rec[4] = {0, 0, 0, 0};
            int64_t lk = 0;
            RGB c = trace_path(s, rng, static_cast<int>(px), static_cast<int>(py), rec, &lk, nrc, item, unbiased);
            total += lk;
            if (dlog) std::memcpy(dlog + 4 * static_cast<size_t>(item), rec, sizeof(rec));
            rng_states[pix] = rng.state;
            if (nrc->mode == 1) {
                if (!all_nonneg_finite(c)) c = rgb(0, 0, 0);
                float* fc = nrc->frame_contribution + 3 * static_cast<size_t>(item);
                fc[0] = c.r;
                fc[1] = c.g;
                fc[2] = c.b;
            }
        }
    }
    return total;
}

}  // extern "C"
