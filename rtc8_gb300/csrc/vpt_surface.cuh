// Device side of the surface path: triangle meshes hit through a BVH (the reference traces them
// with OptiX), surface points, the reference's BSDFs and area-light sampling.
// Citations are file:line within the reference project (shocker-0x15/rtcamp8).
#pragma once

#include "vpt_device.cuh"

namespace vpt {

// Material kinds (include/rtc8_vpt.h VPT_MATERIAL_*).
constexpr int kMatSimplePbr = 0;
constexpr int kMatLambert = 1;

// probToSampleEnvLight (renderer/renderer_shared.h:10).
constexpr float kProbEnvLight = 0.25f;

// BVH node: an axis-aligned box and either two children (count == 0: children `first` and
// `first + 1`) or a leaf of `count` entries of the triangle order starting at `first`.
struct BvhNode {
    float lo[3];
    uint32_t first;
    float hi[3];
    uint32_t count;
};

// An instance: object-to-world transform (row-major 3x4), the 3x3 matrix that carries normals
// (its rows are the columns of the inverse of the transform's linear part), the instance's
// uniform scale, its geometry group and its first placement (one per geometry of the group,
// in group order).
struct SurfInstance {
    float m[12];
    float nm[9];
    float uniform_scale;
    uint32_t group;
    uint32_t first_place;
};

// A geometry group: a contiguous range of geometry instances and its light distribution over
// them (weights = the geometries' emitter integrals).
struct SurfGroup {
    uint32_t first_geom, num_geoms;
    uint32_t dist_off;   // offset of its weights / CDF in Surfaces::group_w / group_cdf
    float integral;
};

// A geometry instance (a mesh with one material): object-space vertices and triangles and the
// distribution over its emitting triangles.
struct SurfGeom {
    uint32_t first_vertex, first_tri, num_tris, material;
    uint32_t prim_off;   // offset of its weights / CDF in Surfaces::prim_w / prim_cdf
    float prim_integral;
};

// Decoded material: the BSDF parameters the reference's setupBSDFBody derives from its 1x1
// textures (common_renderer_types.h:1524-1541, 1962-1985) and the emittance.
struct SurfMaterial {
    float diffuse[3];
    float specular[3];
    float roughness;   // 1 - smoothness
    int32_t kind;
    float emittance[3];
    int32_t emissive;
};

struct Surfaces {
    const BvhNode* __restrict__ nodes;
    const uint32_t* __restrict__ order;      // BVH leaf entries -> world triangle
    const float4* __restrict__ tri_pos;      // 3 world positions per world triangle (w of the first: placement)
    const uint4* __restrict__ places;        // instance, geometry, first world triangle
    const SurfInstance* __restrict__ insts;
    const SurfGroup* __restrict__ groups;
    const SurfGeom* __restrict__ geoms;
    const uint4* __restrict__ obj_tri;       // object-space vertex indices (relative to the geometry)
    const float4* __restrict__ obj_nrm;      // object-space shading normals
    const float4* __restrict__ obj_tan;      // object-space tangents
    const SurfMaterial* __restrict__ mats;
    const float* __restrict__ prim_w;
    const float* __restrict__ prim_cdf;
    const float* __restrict__ group_w;
    const float* __restrict__ group_cdf;
    const float* __restrict__ inst_w;
    const float* __restrict__ inst_cdf;
    uint32_t num_insts;
    uint32_t num_tris;
    float inst_integral;   // lightInstDist.integral(): > 0 when some triangle emits
    int32_t enabled;
};

// ------------------------------------------------------------------------------ helpers
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ V3 ld3(float4 v) { return v3(v.x, v.y, v.z); }
__device__ __forceinline__ float pow5f(float x) {
    const float x2 = x * x;
    return x * (x2 * x2);
}
__device__ __forceinline__ float lerpf(float a, float b, float t) { return (1 - t) * a + t * b; }
__device__ __forceinline__ RGB lerp_rgb(RGB a, RGB b, float t) { return (1 - t) * a + t * b; }

// Matrix4x4 * Vector3D (the 3x3 part, row dot products, basic_types.h:2130-2134).
__device__ __forceinline__ V3 xform_vector(const float* m, V3 v) {
    return v3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
              m[8] * v.x + m[9] * v.y + m[10] * v.z);
}
// StaticTransform * Normal3D (common_renderer_types.h:1080-1085): nm holds the rows it uses.
__device__ __forceinline__ V3 xform_normal(const float* nm, V3 n) {
    return v3(nm[0] * n.x + nm[1] * n.y + nm[2] * n.z, nm[3] * n.x + nm[4] * n.y + nm[5] * n.z,
              nm[6] * n.x + nm[7] * n.y + nm[8] * n.z);
}

// offsetRayOrigin (common_renderer_types.h:1324-1349): Ray Tracing Gems ch. 6, integer offsets
// of the float bit patterns away from the surface, a plain float offset near the origin.
__device__ __forceinline__ float offset_coord(float p, float n) {
    const int32_t oi = static_cast<int32_t>(256.0f * n);
    const float p1 = __int_as_float(__float_as_int(p) + (p < 0 ? -oi : oi));
    const float p2 = p + (1.0f / 65536.0f) * n;
    return fabsf(p) < (1.0f / 32.0f) ? p2 : p1;
}
__device__ __forceinline__ V3 offset_ray_origin(V3 p, V3 n) {
    return v3(offset_coord(p.x, n.x), offset_coord(p.y, n.y), offset_coord(p.z, n.z));
}

// DiscreteDistribution1DTemplate<float, false>::sample (common_renderer_types.h:165-188): binary
// search of the exclusive CDF, probability and the remapped variate.
__device__ __forceinline__ uint32_t dist_sample(const float* w, const float* cdf, uint32_t n, float integral, float u,
                                                float* prob, float* remapped) {
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

// ------------------------------------------------------------------------------ BVH
// Möller-Trumbore in the operation order of the reference's barycentric restoration
// (renderer_kernel_common.h:236-248). Two-sided, hits with t in [tmin, tmax].
__device__ __forceinline__ bool tri_hit(V3 o, V3 d, V3 p0, V3 p1, V3 p2, float tmin, float tmax, float* t, float* b1,
                                        float* b2) {
    const V3 e1 = p1 - p0, e2 = p2 - p0;
    const V3 pv = cross(d, e2);
    const float det = dot(e1, pv);
    if (det == 0.0f) return false;
    const float rdet = 1.0f / det;
    const V3 tv = o - p0;
    const float u = dot(tv, pv) * rdet;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    const V3 qv = cross(tv, e1);
    const float v = dot(d, qv) * rdet;
    if (!(v >= 0.0f && u + v <= 1.0f)) return false;
    const float tt = dot(e2, qv) * rdet;
    if (!(tt >= tmin && tt <= tmax)) return false;
    *t = tt;
    *b1 = u;
    *b2 = v;
    return true;
}

// Entry distance of a ray into a node's box (slab test), +inf when it misses [tmin, tmax].
__device__ __forceinline__ float box_entry(const BvhNode& nd, V3 o, V3 inv, float tmin, float tmax) {
    float t0 = tmin, t1 = tmax;
    const float lo[3] = {nd.lo[0], nd.lo[1], nd.lo[2]};
    const float hi[3] = {nd.hi[0], nd.hi[1], nd.hi[2]};
    const float oo[3] = {o.x, o.y, o.z};
    const float ii[3] = {inv.x, inv.y, inv.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float ta = (lo[a] - oo[a]) * ii[a];
        float tb = (hi[a] - oo[a]) * ii[a];
        if (ta > tb) {
            const float s = ta;
            ta = tb;
            tb = s;
        }
        // NaN (0 * inf on a slab plane) leaves the interval as it is.
        t0 = ta > t0 ? ta : t0;
        t1 = tb < t1 ? tb : t1;
    }
    return t0 <= t1 ? t0 : INFINITY;
}

constexpr int kBvhStack = 64;
// Scenes of at most this many world triangles are not traversed: every lane of a warp tests the
// same triangle in the same step (one broadcast load, no stack, no divergence), which beats a
// tree whose boxes a small scene's large triangles overlap. Hits and ties are the tree's.
constexpr uint32_t kFlatTriangles = 64;

struct SurfHit {
    uint32_t tri;   // world triangle, ~0u = none
    float t, b1, b2;
};

// Closest hit in [tmin, tmax]; ties in t go to the lower world-triangle index (the oracle's
// brute-force search applies the same rule). Sets *overflow if the traversal stack overflowed
// (the builder bounds the depth below the stack size, so trees it built never do).
static __device__ __noinline__ SurfHit bvh_closest(const Surfaces& S, V3 o, V3 d, float tmin, float tmax, bool* overflow) {
    SurfHit h{~0u, tmax, 0.0f, 0.0f};
    if (S.num_tris <= kFlatTriangles) {
        // Ascending index order: a later triangle replaces the best only when strictly closer.
        for (uint32_t tri = 0; tri < S.num_tris; ++tri) {
            float t, b1, b2;
            if (tri_hit(o, d, ld3(S.tri_pos[3 * tri]), ld3(S.tri_pos[3 * tri + 1]), ld3(S.tri_pos[3 * tri + 2]), tmin,
                        h.t, &t, &b1, &b2) &&
                (t < h.t || tri < h.tri)) {
                h.tri = tri;
                h.t = t;
                h.b1 = b1;
                h.b2 = b2;
            }
        }
        return h;
    }
    const V3 inv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    uint32_t stack[kBvhStack];
    int sp = 0;
    if (box_entry(S.nodes[0], o, inv, tmin, tmax) == INFINITY) return h;
    uint32_t node = 0;
    while (true) {
        const BvhNode nd = S.nodes[node];
        if (nd.count > 0) {
            for (uint32_t k = 0; k < nd.count; ++k) {
                const uint32_t tri = S.order[nd.first + k];
                float t, b1, b2;
                if (tri_hit(o, d, ld3(S.tri_pos[3 * tri]), ld3(S.tri_pos[3 * tri + 1]), ld3(S.tri_pos[3 * tri + 2]), tmin,
                            h.t, &t, &b1, &b2) &&
                    (t < h.t || tri < h.tri)) {
                    h.tri = tri;
                    h.t = t;
                    h.b1 = b1;
                    h.b2 = b2;
                }
            }
        } else {
            const uint32_t a = nd.first, b = nd.first + 1;
            const float ta = box_entry(S.nodes[a], o, inv, tmin, h.t);
            const float tb = box_entry(S.nodes[b], o, inv, tmin, h.t);
            const bool ha = ta != INFINITY, hb = tb != INFINITY;
            if (ha && hb) {
                const uint32_t nearc = ta <= tb ? a : b, farc = ta <= tb ? b : a;
                if (sp < kBvhStack) {
                    stack[sp++] = farc;
                } else {
                    *overflow = true;
                }
                node = nearc;
                continue;
            }
            if (ha || hb) {
                node = ha ? a : b;
                continue;
            }
        }
        // Next pending node that the current closest hit does not exclude.
        bool found = false;
        while (sp > 0) {
            const uint32_t n2 = stack[--sp];
            if (box_entry(S.nodes[n2], o, inv, tmin, h.t) != INFINITY) {
                node = n2;
                found = true;
                break;
            }
        }
        if (!found) break;
    }
    return h;
}

// Any hit in [tmin, tmax] (the visibility ray's any-hit program, optix_pathtracing_kernels.cu:7-10).
static __device__ __noinline__ bool bvh_any(const Surfaces& S, V3 o, V3 d, float tmin, float tmax, bool* overflow) {
    if (S.num_tris <= kFlatTriangles) {
        for (uint32_t tri = 0; tri < S.num_tris; ++tri) {
            float t, b1, b2;
            if (tri_hit(o, d, ld3(S.tri_pos[3 * tri]), ld3(S.tri_pos[3 * tri + 1]), ld3(S.tri_pos[3 * tri + 2]), tmin,
                        tmax, &t, &b1, &b2))
                return true;
        }
        return false;
    }
    const V3 inv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    uint32_t stack[kBvhStack];
    int sp = 0;
    if (box_entry(S.nodes[0], o, inv, tmin, tmax) == INFINITY) return false;
    stack[sp++] = 0;
    while (sp > 0) {
        const BvhNode nd = S.nodes[stack[--sp]];
        if (nd.count > 0) {
            for (uint32_t k = 0; k < nd.count; ++k) {
                const uint32_t tri = S.order[nd.first + k];
                float t, b1, b2;
                if (tri_hit(o, d, ld3(S.tri_pos[3 * tri]), ld3(S.tri_pos[3 * tri + 1]), ld3(S.tri_pos[3 * tri + 2]), tmin,
                            tmax, &t, &b1, &b2))
                    return true;
            }
        } else {
            for (uint32_t c = nd.first; c < nd.first + 2; ++c) {
                if (box_entry(S.nodes[c], o, inv, tmin, tmax) == INFINITY) continue;
                if (sp < kBvhStack) {
                    stack[sp++] = c;
                } else {
                    *overflow = true;
                }
            }
        }
    }
    return false;
}

// ------------------------------------------------------------------------------ surface point
struct SurfPoint {
    V3 pos;
    V3 gn;          // geometric normal (unit)
    Frame sf;       // shading frame: tangent, bitangent = cross(normal, tangent), normal
    float hyp_area_pdf;
    uint32_t material;
};

// computeSurfacePoint (renderer_kernel_common.h:72-124) for world triangle `tri` at (b1, b2).
// `env_enabled`: the environment takes probToSampleEnvLight of the light selection.
static __device__ __noinline__ SurfPoint surface_point(const Surfaces& S, uint32_t tri, float b1, float b2,
                                                   bool env_enabled) {
    const float4 q0 = S.tri_pos[3 * tri];
    const V3 p0 = ld3(q0), p1 = ld3(S.tri_pos[3 * tri + 1]), p2 = ld3(S.tri_pos[3 * tri + 2]);
    const uint4 pl = S.places[__float_as_uint(q0.w)];
    const SurfInstance& in = S.insts[pl.x];
    const SurfGeom& ge = S.geoms[pl.y];
    const uint32_t prim = tri - pl.z;
    const uint4 vi = S.obj_tri[ge.first_tri + prim];
    const float b0 = 1 - (b1 + b2);
    SurfPoint sp;
    sp.pos = b0 * p0 + b1 * p1 + b2 * p2;
    const V3 gn = cross(p1 - p0, p2 - p0);
    const float area = 0.5f * sqrtf(dot(gn, gn));
    const float rg = 1.0f / (2 * area);
    sp.gn = gn * rg;
    const V3 n0 = ld3(S.obj_nrm[ge.first_vertex + vi.x]), n1 = ld3(S.obj_nrm[ge.first_vertex + vi.y]),
             n2 = ld3(S.obj_nrm[ge.first_vertex + vi.z]);
    const V3 t0 = ld3(S.obj_tan[ge.first_vertex + vi.x]), t1 = ld3(S.obj_tan[ge.first_vertex + vi.y]),
             t2 = ld3(S.obj_tan[ge.first_vertex + vi.z]);
    const V3 ln = b0 * n0 + b1 * n1 + b2 * n2;
    const V3 lt = b0 * t0 + b1 * t1 + b2 * t2;
    sp.sf.n = normalize(xform_normal(in.nm, ln));
    sp.sf.t = normalize(xform_vector(in.m, lt));
    sp.sf.b = cross(sp.sf.n, sp.sf.t);
    sp.material = ge.material;
    // :103-123: probability density of reaching this point by area-light sampling.
    float light_prob = 1.0f;
    if (env_enabled) light_prob *= (1 - kProbEnvLight);
    const SurfGroup& gr = S.groups[in.group];
    const float group_imp = gr.integral;
    const float inst_imp = (in.uniform_scale * in.uniform_scale) * group_imp;
    sp.hyp_area_pdf = 0.0f;
    if (S.inst_integral > 0.0f) {
        const float inst_prob = inst_imp / S.inst_integral;
        if (!(inst_prob == 0.0f)) {
            light_prob *= inst_prob;
            const float geom_prob = ge.prim_integral / group_imp;
            if (!(geom_prob == 0.0f)) {
                light_prob *= geom_prob;
                const float pmf = ge.prim_integral == 0.0f ? 0.0f : S.prim_w[ge.prim_off + prim] / ge.prim_integral;
                light_prob *= pmf;
                sp.hyp_area_pdf = light_prob / area;
            }
        }
    }
    return sp;
}

// ------------------------------------------------------------------------------ BSDFs
// concentricSampleDisk + cosineSampleHemisphere (common_renderer_types.h:1265-1307).
__device__ __forceinline__ V3 cosine_sample_hemisphere(float u0, float u1) {
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
        } else {
            if (sx > sy) {
                r = -sy;
                th = 6 + sx / sy;
            } else {
                r = -sx;
                th = 4 + sy / sx;
            }
        }
        th *= kPi / 4;
        x = r * cosf(th);
        y = r * sinf(th);
    }
    return v3(x, y, sqrtf(fmaxf(0.0f, 1.0f - x * x - y * y)));
}

// GGX with height-correlated Smith masking (common_renderer_types.h:1595-1650).
__device__ __forceinline__ float ggx_d(float ag, V3 m) {
    if (m.z <= 0.0f) return 0.0f;
    const float tmp = m.x * m.x + m.y * m.y + (m.z * ag) * (m.z * ag);
    return (ag * ag) / (kPi * (tmp * tmp));
}
__device__ __forceinline__ float ggx_g1(float ag, V3 v, V3 m) {
    if (dot(v, m) * v.z <= 0) return 0.0f;
    const float tmp = (ag * ag) * (v.x * v.x + v.y * v.y) / (v.z * v.z);
    return 2 / (1 + sqrtf(1 + tmp));
}
__device__ __forceinline__ float ggx_g_hc(float ag, V3 v1, V3 v2, V3 m) {
    const float a1 = (ag * ag) * (v1.x * v1.x + v1.y * v1.y) / (v1.z * v1.z);
    const float a2 = (ag * ag) * (v2.x * v2.x + v2.y * v2.y) / (v2.z * v2.z);
    const float l1 = (-1 + sqrtf(1 + a1)) / 2;
    const float l2 = (-1 + sqrtf(1 + a2)) / 2;
    const float c1 = (dot(v1, m) / v1.z) > 0 ? 1.0f : 0.0f;
    const float c2 = (dot(v2, m) / v2.z) > 0 ? 1.0f : 0.0f;
    return c1 * c2 / (1 + l1 + l2);
}
__device__ __forceinline__ float ggx_pdf(float ag, V3 v, V3 m) {
    return ggx_g1(ag, v, m) * fabsf(dot(v, m)) * ggx_d(ag, m) / fabsf(v.z);
}
// Visible-normal sampling of the stretched GGX (common_renderer_types.h:1618-1646).
__device__ __forceinline__ float ggx_sample(float ag, V3 v, float u0, float u1, V3* m, float* m_pdf) {
    const V3 sv = normalize(v3(ag * v.x, ag * v.y, v.z));
    const float dist2d = sqrtf(sv.x * sv.x + sv.y * sv.y);
    const float rd = 1.0f / dist2d;
    const V3 T1 = (sv.z < 0.9999f) ? v3(sv.y * rd, -sv.x * rd, 0) : v3(1, 0, 0);
    const V3 T2 = v3(T1.y * sv.z, -T1.x * sv.z, dist2d);
    const float a = 1.0f / (1.0f + sv.z);
    const float r = sqrtf(u0);
    const float phi = kPi * ((u1 < a) ? u1 / a : 1 + (u1 - a) / (1.0f - a));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    const float P1 = r * cp;
    const float P2 = r * sp * ((u1 < a) ? 1.0f : sv.z);
    V3 mm = P1 * T1 + P2 * T2 + sqrtf(1.0f - P1 * P1 - P2 * P2) * sv;
    mm = normalize(v3(ag * mm.x, ag * mm.y, mm.z));
    *m = mm;
    const float D = ggx_d(ag, mm);
    *m_pdf = ggx_g1(ag, v, mm) * fabsf(dot(v, mm)) * D / fabsf(v.z);
    return D;
}

struct Bsdf {
    RGB diffuse, specular;
    float roughness;
    int32_t kind;
};
__device__ __forceinline__ Bsdf make_bsdf(const SurfMaterial& m) {
    return Bsdf{rgb(m.diffuse[0], m.diffuse[1], m.diffuse[2]), rgb(m.specular[0], m.specular[1], m.specular[2]),
                m.roughness, m.kind};
}

// Selection weights of the dichromatic BRDF's two lobes (:1690-1705 / :1850-1865, the
// non-fitted form the reference compiles).
__device__ __forceinline__ void dichromatic_weights(const Bsdf& f, float qz, float vz, float* wd, float* ws) {
    const float one_minus_vn5 = pow5f(1 - vz);
    const float fd90 = 0.5f * f.roughness + 2 * f.roughness * qz * qz;
    const float edf = lerpf(1.0f, fd90, one_minus_vn5);
    *wd = luminance(f.diffuse) * (edf * edf) * lerpf(1.0f, 1.0f / 1.51f, f.roughness);
    const float evh5 = pow5f(1 - vz);
    *ws = lerpf(luminance(f.specular), 1.0f, evh5);
}

// The dichromatic value for the light direction L and view V (both in the upper hemisphere),
// microfacet normal m (:1760-1785 / :1801-1826).
__device__ __forceinline__ RGB dichromatic_value(const Bsdf& f, float ag, V3 L, V3 V, V3 m, float dot_lh, float D) {
    const float one_minus_lh5 = pow5f(1 - dot_lh);
    const float G = ggx_g_hc(ag, L, V, m);
    const RGB F = lerp_rgb(f.specular, rgb(1.0f, 1.0f, 1.0f), one_minus_lh5);
    const float denom = 4 * L.z * V.z;
    RGB spec = F * ((D * G) / denom);
    if (G == 0) spec = rgb(0, 0, 0);
    const float fd90 = 0.5f * f.roughness + 2 * f.roughness * dot_lh * dot_lh;
    const float one_minus_vn5 = pow5f(1 - V.z);
    const float one_minus_ln5 = pow5f(1 - L.z);
    const float fout = lerpf(1.0f, fd90, one_minus_vn5);
    const float fin = lerpf(1.0f, fd90, one_minus_ln5);
    const RGB diff = f.diffuse * (fout * fin * lerpf(1.0f, 1.0f / 1.51f, f.roughness) / kPi);
    return diff + spec;
}

// BSDF::sampleF (Lambert :1497-1505, dichromatic :1680-1790). `q` = the query direction (vOut)
// in the shading frame. Returns the value; *pdf = 0 marks a failed sample.
static __device__ __noinline__ RGB bsdf_sample(const Bsdf& f, V3 q, float u0, float u1, V3* out, float* pdf) {
    if (f.kind == kMatLambert) {
        V3 d = cosine_sample_hemisphere(u0, u1);
        *pdf = d.z / kPi;
        if (q.z <= 0.0f) d.z *= -1;
        *out = d;
        return rdiv(f.diffuse, kPi);
    }
    const float ag = f.roughness * f.roughness;
    const bool entering = q.z >= 0.0f;
    const V3 V = entering ? q : -q;
    float wd, ws;
    dichromatic_weights(f, q.z, V.z, &wd, &ws);
    const float sum = wd + ws;
    if (sum == 0.0f) {
        *pdf = 0.0f;
        return rgb(0, 0, 0);
    }
    float ud1 = u1;
    const float uc = ud1;
    float pdf_d, pdf_s, dot_lh, D;
    V3 L, m;
    if (sum * uc < wd) {
        ud1 = (sum * uc - 0) / wd;
        L = cosine_sample_hemisphere(u0, ud1);
        pdf_d = L.z / kPi;
        m = normalize(L + V);
        dot_lh = fminf(dot(L, m), 1.0f);
        const float common = 1.0f / (4 * dot_lh);
        pdf_s = common * ggx_pdf(ag, V, m);
        D = ggx_d(ag, m);
    } else {
        ud1 = (sum * uc - wd) / ws;
        float m_pdf;
        D = ggx_sample(ag, V, u0, ud1, &m, &m_pdf);
        const float dot_vh = fminf(dot(V, m), 1.0f);
        dot_lh = dot_vh;
        L = (2 * dot_vh) * m - V;
        if (L.z * V.z <= 0) {
            *pdf = 0.0f;
            return rgb(0, 0, 0);
        }
        const float common = 1.0f / (4 * dot_lh);
        pdf_s = common * m_pdf;
        pdf_d = L.z / kPi;
    }
    const RGB val = dichromatic_value(f, ag, L, V, m, dot_lh, D);
    *out = entering ? L : -L;
    *pdf = (pdf_d * wd + pdf_s * ws) / sum;
    return val;
}

// BSDF::evaluateF (Lambert :1506-1511, dichromatic :1792-1829).
__device__ __forceinline__ RGB bsdf_eval(const Bsdf& f, V3 q, V3 s) {
    if (f.kind == kMatLambert) return (q.z * s.z > 0) ? rdiv(f.diffuse, kPi) : rgb(0, 0, 0);
    const float ag = f.roughness * f.roughness;
    if (s.z * q.z <= 0) return rgb(0, 0, 0);
    const bool entering = q.z >= 0.0f;
    const V3 V = entering ? q : -q;
    const V3 L = entering ? s : -s;
    const V3 m = normalize(L + V);
    const float dot_lh = dot(L, m);
    return dichromatic_value(f, ag, L, V, m, dot_lh, ggx_d(ag, m));
}

// evaluateF and evaluatePDF of one direction together (NEE needs both), out of line.
__device__ __forceinline__ float bsdf_pdf(const Bsdf& f, V3 q, V3 s);
static __device__ __noinline__ RGB bsdf_eval_pdf(const Bsdf& f, V3 q, V3 s, float* pdf);

// BSDF::evaluatePDF (Lambert :1512-1517, dichromatic :1830-1875).
__device__ __forceinline__ float bsdf_pdf(const Bsdf& f, V3 q, V3 s) {
    if (f.kind == kMatLambert) return (q.z * s.z > 0) ? fabsf(s.z) / kPi : 0.0f;
    const float ag = f.roughness * f.roughness;
    const bool entering = q.z >= 0.0f;
    const V3 V = entering ? q : -q;
    const V3 L = entering ? s : -s;
    const V3 m = normalize(L + V);
    const float dot_lh = dot(L, m);
    const float common = 1.0f / (4 * dot_lh);
    float wd, ws;
    dichromatic_weights(f, q.z, V.z, &wd, &ws);
    const float sum = wd + ws;
    if (sum == 0.0f) return 0.0f;
    const float pd = L.z / kPi;
    const float ps = common * ggx_pdf(ag, V, m);
    return (pd * wd + ps * ws) / sum;
}

// ------------------------------------------------------------------------------ area lights
struct AreaSample {
    V3 pos, normal;
    RGB emittance;
    float area_pdf;   // 0: no sample
};

// sampleLight<false> for the area lights (renderer_kernel_common.h:146-290): instance, geometry
// of its group, triangle (each a CDF search that remaps the variate for the next level), then a
// uniform point by the low-distortion triangle map.
static __device__ __noinline__ AreaSample sample_area_light(const Surfaces& S, float ul, float u0, float u1) {
    AreaSample a;
    a.area_pdf = 0.0f;
    a.emittance = rgb(0, 0, 0);
    a.pos = a.normal = v3(0, 0, 0);
    float light_prob = 1.0f;
    float inst_prob, u_geom;
    const uint32_t ii = dist_sample(S.inst_w, S.inst_cdf, S.num_insts, S.inst_integral, ul, &inst_prob, &u_geom);
    light_prob *= inst_prob;
    if (inst_prob == 0.0f) return a;
    const SurfInstance& in = S.insts[ii];
    const SurfGroup& gr = S.groups[in.group];
    float geom_prob, u_prim;
    const uint32_t gi = dist_sample(S.group_w + gr.dist_off, S.group_cdf + gr.dist_off, gr.num_geoms, gr.integral,
                                    u_geom, &geom_prob, &u_prim);
    light_prob *= geom_prob;
    if (geom_prob == 0.0f) return a;
    const SurfGeom& ge = S.geoms[gr.first_geom + gi];
    float prim_prob, unused;
    const uint32_t prim = dist_sample(S.prim_w + ge.prim_off, S.prim_cdf + ge.prim_off, ge.num_tris, ge.prim_integral,
                                      u_prim, &prim_prob, &unused);
    light_prob *= prim_prob;
    const uint4 pl = S.places[in.first_place + gi];
    const uint32_t tri = pl.z + prim;
    const V3 p0 = ld3(S.tri_pos[3 * tri]), p1 = ld3(S.tri_pos[3 * tri + 1]), p2 = ld3(S.tri_pos[3 * tri + 2]);
    const V3 gnv = cross(p1 - p0, p2 - p0);
    float t0 = 0.5f * u0, t1 = 0.5f * u1;
    const float off = t1 - t0;
    if (off > 0)
        t1 += off;
    else
        t0 -= off;
    const float t2 = 1 - (t0 + t1);
    const float rec_area = 2.0f / sqrtf(dot(gnv, gnv));
    a.area_pdf = light_prob * rec_area;
    a.pos = t0 * p0 + t1 * p1 + t2 * p2;
    const uint4 vi = S.obj_tri[ge.first_tri + prim];
    const V3 n0 = ld3(S.obj_nrm[ge.first_vertex + vi.x]), n1 = ld3(S.obj_nrm[ge.first_vertex + vi.y]),
             n2 = ld3(S.obj_nrm[ge.first_vertex + vi.z]);
    a.normal = normalize(xform_normal(in.nm, t0 * n0 + t1 * n1 + t2 * n2));
    const SurfMaterial& mt = S.mats[ge.material];
    if (mt.emissive) a.emittance = rgb(mt.emittance[0], mt.emittance[1], mt.emittance[2]);
    return a;
}

static __device__ __noinline__ RGB bsdf_eval_pdf(const Bsdf& f, V3 q, V3 s, float* pdf) {
    *pdf = bsdf_pdf(f, q, s);
    return bsdf_eval(f, q, s);
}

}  // namespace vpt
