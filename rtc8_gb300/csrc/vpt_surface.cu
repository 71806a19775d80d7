// Host side of the surface path: scene arrays, the BVH and the light distributions of the
// emitting triangles (vpt_set_surfaces), replacing the reference's OptiX geometry set-up
// (renderer/renderer_scene.cpp:227-352) and its light-probability kernels
// (renderer/gpu_kernels/compute_light_probs.cu:19-157, renderer_scene.cpp:353-468).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "vpt_ctx.h"
#include "vpt_surface.cuh"

namespace vpt {
namespace {

int fail(int code, const std::string& msg) { return ctx_set_error(code, msg.c_str()); }

// Binned-SAH BVH over world triangles. Leaves hold at most kLeafMax triangles unless the depth
// limit forces a leaf; the depth limit keeps the device traversal stack (kBvhStack) sufficient.
constexpr int kLeafMax = 4;
constexpr int kBins = 16;
constexpr int kMaxDepth = 48;
static_assert(kMaxDepth < kBvhStack, "the traversal stack must hold one entry per level");

struct Box {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void add(const float* p) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    void add(const Box& b) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    double half_area() const {
        double d[3];
        for (int a = 0; a < 3; ++a) d[a] = std::max(0.0, static_cast<double>(hi[a]) - lo[a]);
        return d[0] * d[1] + d[1] * d[2] + d[2] * d[0];
    }
};

struct BuildTask {
    uint32_t node, begin, end;
    int depth;
};

int bin_of(float c, float lo, double scale) {
    const int b = static_cast<int>((c - lo) * scale);
    return std::min(std::max(b, 0), kBins - 1);
}

void build_bvh(const std::vector<float>& pos, uint32_t ntri, std::vector<BvhNode>* nodes_out,
               std::vector<uint32_t>* order_out) {
    std::vector<Box> tb(ntri);
    std::vector<float> cen(3 * static_cast<size_t>(ntri));
    Box scene;
    for (uint32_t t = 0; t < ntri; ++t) {
        for (int k = 0; k < 3; ++k) tb[t].add(&pos[9 * static_cast<size_t>(t) + 3 * k]);
        for (int a = 0; a < 3; ++a) cen[3 * static_cast<size_t>(t) + a] = 0.5f * (tb[t].lo[a] + tb[t].hi[a]);
        scene.add(tb[t]);
    }
    // Boxes grow by a margin of the scene's size, so that a hit on a triangle lying in a box face
    // is never excluded by the rounding of the slab test.
    double diag = 0, mag = 0;
    for (int a = 0; a < 3; ++a) {
        diag = std::max(diag, static_cast<double>(scene.hi[a]) - scene.lo[a]);
        mag = std::max({mag, std::fabs(static_cast<double>(scene.lo[a])), std::fabs(static_cast<double>(scene.hi[a]))});
    }
    const float pad = static_cast<float>(1e-5 * diag + 1e-6 * mag + 1e-30);

    std::vector<uint32_t>& order = *order_out;
    order.resize(ntri);
    for (uint32_t t = 0; t < ntri; ++t) order[t] = t;
    std::vector<BvhNode>& nodes = *nodes_out;
    nodes.clear();
    nodes.push_back(BvhNode{});
    std::vector<BuildTask> stack{{0, 0, ntri, 0}};
    while (!stack.empty()) {
        const BuildTask task = stack.back();
        stack.pop_back();
        Box bb, cb;
        for (uint32_t i = task.begin; i < task.end; ++i) {
            bb.add(tb[order[i]]);
            cb.add(&cen[3 * static_cast<size_t>(order[i])]);
        }
        for (int a = 0; a < 3; ++a) {
            nodes[task.node].lo[a] = bb.lo[a] - pad;
            nodes[task.node].hi[a] = bb.hi[a] + pad;
        }
        const uint32_t n = task.end - task.begin;
        int best_axis = -1, best_bin = 0;
        double best_cost = static_cast<double>(n);  // cost of a leaf, in triangle tests
        if (n > kLeafMax && task.depth < kMaxDepth) {
            const double parent = std::max(bb.half_area(), 1e-30);
            for (int a = 0; a < 3; ++a) {
                const float lo = cb.lo[a], hi = cb.hi[a];
                if (!(hi > lo)) continue;
                Box bins[kBins];
                uint32_t count[kBins] = {};
                const double scale = kBins / (static_cast<double>(hi) - lo);
                for (uint32_t i = task.begin; i < task.end; ++i) {
                    const uint32_t t = order[i];
                    const int b = bin_of(cen[3 * static_cast<size_t>(t) + a], lo, scale);
                    ++count[b];
                    bins[b].add(tb[t]);
                }
                Box left[kBins];
                uint32_t lc[kBins];
                Box acc;
                uint32_t c = 0;
                for (int b = 0; b < kBins; ++b) {
                    acc.add(bins[b]);
                    c += count[b];
                    left[b] = acc;
                    lc[b] = c;
                }
                Box racc;
                uint32_t rc = 0;
                for (int b = kBins - 1; b >= 1; --b) {
                    racc.add(bins[b]);
                    rc += count[b];
                    const uint32_t lcount = lc[b - 1];
                    if (lcount == 0 || rc == 0) continue;
                    const double cost = 0.125 + (left[b - 1].half_area() * lcount + racc.half_area() * rc) / parent;
                    if (cost < best_cost) {
                        best_cost = cost;
                        best_axis = a;
                        best_bin = b;
                    }
                }
            }
        }
        uint32_t mid = 0;
        if (best_axis >= 0) {
            const float lo = cb.lo[best_axis], hi = cb.hi[best_axis];
            const double scale = kBins / (static_cast<double>(hi) - lo);
            auto it = std::partition(order.begin() + task.begin, order.begin() + task.end, [&](uint32_t t) {
                return bin_of(cen[3 * static_cast<size_t>(t) + best_axis], lo, scale) < best_bin;
            });
            mid = static_cast<uint32_t>(it - order.begin());
            if (mid == task.begin || mid == task.end) best_axis = -1;
        } else if (n > kLeafMax && task.depth < kMaxDepth && best_cost >= static_cast<double>(n) &&
                   !(cb.hi[0] > cb.lo[0]) && !(cb.hi[1] > cb.lo[1]) && !(cb.hi[2] > cb.lo[2])) {
            // All centroids coincide: split the range in halves.
            mid = task.begin + n / 2;
            best_axis = 3;
        }
        if (best_axis < 0) {
            nodes[task.node].first = task.begin;
            nodes[task.node].count = n;
            continue;
        }
        const uint32_t child = static_cast<uint32_t>(nodes.size());
        nodes[task.node].first = child;
        nodes[task.node].count = 0;
        nodes.push_back(BvhNode{});
        nodes.push_back(BvhNode{});
        stack.push_back({child, task.begin, mid, task.depth + 1});
        stack.push_back({child + 1, mid, task.end, task.depth + 1});
    }
}

// Immediate colour of the reference's 1x1 textures: 8-bit (truncated, renderer_scene.cpp:
// 860-900), read back with the sRGB decode when the texture is a colour.
float unorm8(float v) {
    const float s = 255.0f * v;
    const uint32_t q = std::min<uint32_t>(s > 0.0f ? static_cast<uint32_t>(s) : 0u, 255u);
    return static_cast<float>(q);
}
float srgb_decode8(float v) {
    const double c = unorm8(v) / 255.0;
    return static_cast<float>(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
}
float linear8(float v) { return unorm8(v) / 255.0f; }

float luminance3(const float* c) { return 0.2126729f * c[0] + 0.7151522f * c[1] + 0.0721750f * c[2]; }

template <typename T, typename Ptr>
int upload(VptContextImpl* c, const std::vector<T>& v, Ptr* out) {
    void* p = nullptr;
    const size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) return fail(VPT_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    c->surf_mem.push_back(p);
    if (!v.empty()) {
        e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(VPT_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
    }
    *out = static_cast<const T*>(p);
    return VPT_OK;
}

// Exclusive prefix sums of `w` (sequential float sums) and the distribution's integral
// (last CDF value + last weight, DiscreteDistribution1D::finalize). The reference forms the CDF
// with a parallel device scan, whose summation order may differ in the last bits.
float exclusive_cdf(const float* w, uint32_t n, float* cdf) {
    float acc = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        cdf[i] = acc;
        acc = acc + w[i];
    }
    return n > 0 ? cdf[n - 1] + w[n - 1] : 0.0f;
}

// Inverse of the linear part of a row-major 3x4 transform, in double.
bool invert3(const float* m, double out[9]) {
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const double det = a * A + b * B + c * C;
    if (!(std::fabs(det) > 0) || !std::isfinite(det)) return false;
    const double r = 1.0 / det;
    out[0] = A * r;
    out[1] = -(b * i - c * h) * r;
    out[2] = (b * f - c * e) * r;
    out[3] = B * r;
    out[4] = (a * i - c * g) * r;
    out[5] = -(a * f - c * d) * r;
    out[6] = C * r;
    out[7] = -(a * h - b * g) * r;
    out[8] = (a * e - b * d) * r;
    return true;
}

// Matrix4x4 * Point3D with w = 1 (basic_types.h:2351-2356), host copy of the device formula.
void xform_point_h(const float* M, const float* p, float* w) {
    w[0] = M[0] * p[0] + M[1] * p[1] + M[2] * p[2] + M[3] * 1.0f;
    w[1] = M[4] * p[0] + M[5] * p[1] + M[6] * p[2] + M[7] * 1.0f;
    w[2] = M[8] * p[0] + M[9] * p[1] + M[10] * p[2] + M[11] * 1.0f;
}

int set_surfaces(VptContextImpl* c, const VptSurfaceMaterial* mats, uint32_t nmat, const VptSurfaceGeometry* geoms,
                 uint32_t ngeom, const VptSurfaceInstance* insts, uint32_t ninst) {
    c->release_surfaces();
    if (ninst == 0) {
        c->update_world_box();
        return VPT_OK;
    }
    if (!mats || !geoms || !insts || nmat == 0 || ngeom == 0)
        return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: null arrays or no materials/geometries");
    constexpr uint64_t kMaxTris = 1ull << 28;
    // Materials.
    std::vector<SurfMaterial> dmat(nmat);
    for (uint32_t k = 0; k < nmat; ++k) {
        const VptSurfaceMaterial& m = mats[k];
        SurfMaterial& d = dmat[k];
        if (m.kind != VPT_MATERIAL_SIMPLE_PBR && m.kind != VPT_MATERIAL_LAMBERT)
            return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: unknown material kind");
        for (int a = 0; a < 3; ++a) {
            if (!std::isfinite(m.base_color[a]) || !std::isfinite(m.emittance[a]) || m.emittance[a] < 0)
                return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: material values must be finite, emittance >= 0");
        }
        if (!std::isfinite(m.roughness) || !std::isfinite(m.metallic))
            return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: material values must be finite");
        float base[3];
        for (int a = 0; a < 3; ++a) base[a] = srgb_decode8(m.base_color[a]);
        d.kind = m.kind;
        if (m.kind == VPT_MATERIAL_LAMBERT) {
            // setupBSDFBody<LambertBRDF> (common_renderer_types.h:1524-1541).
            for (int a = 0; a < 3; ++a) {
                d.diffuse[a] = base[a];
                d.specular[a] = 0.0f;
            }
            d.roughness = 1.0f;
        } else {
            // setupBSDFBody<SimplePBR_BRDF> and its constructor (:1924-1933, 1962-1985), reflectance 0.5.
            const float rough = linear8(m.roughness), metallic = linear8(m.metallic);
            const float smoothness = std::min(1.0f - rough, 0.999f);
            const float reflectance = 0.5f;
            for (int a = 0; a < 3; ++a) {
                d.diffuse[a] = base[a] * (1 - metallic);
                d.specular[a] = 0.16f * (reflectance * reflectance) * (1 - metallic) + base[a] * metallic;
            }
            d.roughness = 1 - smoothness;
        }
        d.emissive = (m.emittance[0] != 0.0f || m.emittance[1] != 0.0f || m.emittance[2] != 0.0f) ? 1 : 0;
        for (int a = 0; a < 3; ++a) d.emittance[a] = m.emittance[a];
    }
    // Geometries: object-space attributes, per-triangle emitter weights and their CDFs.
    std::vector<SurfGeom> dgeom(ngeom);
    std::vector<uint4> obj_tri;
    std::vector<float4> obj_nrm, obj_tan;
    std::vector<float> prim_w, prim_cdf;
    std::vector<Box> geom_box(ngeom);
    uint64_t total_obj_tris = 0, total_obj_verts = 0;
    for (uint32_t g = 0; g < ngeom; ++g) {
        const VptSurfaceGeometry& G = geoms[g];
        if (!G.vertices || !G.triangles || G.num_vertices == 0 || G.num_triangles == 0 || G.material >= nmat)
            return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: geometry without vertices/triangles or bad material");
        total_obj_tris += G.num_triangles;
        total_obj_verts += G.num_vertices;
        if (total_obj_tris > kMaxTris || total_obj_verts > kMaxTris)
            return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: more than 2^28 triangles or vertices");
        SurfGeom& d = dgeom[g];
        d.first_vertex = static_cast<uint32_t>(obj_nrm.size());
        d.first_tri = static_cast<uint32_t>(obj_tri.size());
        d.num_tris = G.num_triangles;
        d.material = G.material;
        d.prim_off = static_cast<uint32_t>(prim_w.size());
        for (uint32_t v = 0; v < G.num_vertices; ++v) {
            const float* a = G.vertices + 9 * static_cast<size_t>(v);
            for (int k = 0; k < 9; ++k)
                if (!std::isfinite(a[k])) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: non-finite vertex");
            geom_box[g].add(a);
            obj_nrm.push_back(make_float4(a[3], a[4], a[5], 0.0f));
            obj_tan.push_back(make_float4(a[6], a[7], a[8], 0.0f));
        }
        const SurfMaterial& mt = dmat[G.material];
        for (uint32_t t = 0; t < G.num_triangles; ++t) {
            const uint32_t* ix = G.triangles + 3 * static_cast<size_t>(t);
            if (ix[0] >= G.num_vertices || ix[1] >= G.num_vertices || ix[2] >= G.num_vertices)
                return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: triangle index out of range");
            obj_tri.push_back(make_uint4(ix[0], ix[1], ix[2], 0u));
            // computeTriangleImportance (compute_light_probs.cu:19-50): object-space area times the
            // luminance of the emittance averaged over the three vertices.
            const float* p0 = G.vertices + 9 * static_cast<size_t>(ix[0]);
            const float* p1 = G.vertices + 9 * static_cast<size_t>(ix[1]);
            const float* p2 = G.vertices + 9 * static_cast<size_t>(ix[2]);
            const float e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
            const float e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
            const float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            const float area = 0.5f * std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            float est[3] = {0.0f, 0.0f, 0.0f};
            if (mt.emissive) {
                for (int k = 0; k < 3; ++k)
                    for (int a = 0; a < 3; ++a) est[a] = est[a] + mt.emittance[a];
                const float third = 1.0f / 3;
                for (int a = 0; a < 3; ++a) est[a] = est[a] * third;
            }
            prim_w.push_back(luminance3(est) * area);
        }
        prim_cdf.resize(prim_w.size());
        d.prim_integral = exclusive_cdf(prim_w.data() + d.prim_off, d.num_tris, prim_cdf.data() + d.prim_off);
    }
    // Groups (one per distinct geometry range of the instances), their distributions over the
    // geometries (computeGeomInstProbBuffer, :53-79) and the instances (computeInstProbBuffer,
    // :82-137: importance = (first column length of the transform)^2 x the group's integral).
    std::vector<SurfGroup> dgroup;
    std::vector<float> group_w, group_cdf;
    std::vector<SurfInstance> dinst(ninst);
    std::vector<uint4> places;
    std::vector<float> tri_pos_f;   // 9 floats per world triangle (BVH build)
    std::vector<float4> tri_pos;
    std::vector<float> inst_w(ninst), inst_cdf(ninst);
    Box world;
    uint64_t world_tris = 0;
    uint32_t emitters = 0;
    for (uint32_t i = 0; i < ninst; ++i) {
        const VptSurfaceInstance& I = insts[i];
        if (I.num_geometries == 0 || static_cast<uint64_t>(I.first_geometry) + I.num_geometries > ngeom)
            return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: instance geometry range out of bounds");
        for (int k = 0; k < 12; ++k)
            if (!std::isfinite(I.transform[k])) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: non-finite transform");
        if (!std::isfinite(I.uniform_scale))
            return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: non-finite uniform scale");
        uint32_t gidx = 0;
        for (; gidx < dgroup.size(); ++gidx)
            if (dgroup[gidx].first_geom == I.first_geometry && dgroup[gidx].num_geoms == I.num_geometries) break;
        if (gidx == dgroup.size()) {
            SurfGroup gr;
            gr.first_geom = I.first_geometry;
            gr.num_geoms = I.num_geometries;
            gr.dist_off = static_cast<uint32_t>(group_w.size());
            for (uint32_t k = 0; k < I.num_geometries; ++k) group_w.push_back(dgeom[I.first_geometry + k].prim_integral);
            group_cdf.resize(group_w.size());
            gr.integral = exclusive_cdf(group_w.data() + gr.dist_off, gr.num_geoms, group_cdf.data() + gr.dist_off);
            dgroup.push_back(gr);
        }
        SurfInstance& d = dinst[i];
        std::memcpy(d.m, I.transform, sizeof(d.m));
        double inv[9];
        if (!invert3(I.transform, inv)) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: singular transform");
        // Normal rows: (inv00, inv10, inv20), (inv01, inv11, inv21), (inv02, inv12, inv22).
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) d.nm[3 * r + k] = static_cast<float>(inv[3 * k + r]);
        d.uniform_scale = I.uniform_scale;
        d.group = gidx;
        d.first_place = static_cast<uint32_t>(places.size());
        const float* M = I.transform;
        const float col0 = std::sqrt(M[0] * M[0] + M[4] * M[4] + M[8] * M[8]);
        inst_w[i] = (col0 * col0) * dgroup[gidx].integral;
        // World box of the instance: the group's object box, 8 corners transformed (basic_types.h:2876-2888).
        Box gb;
        for (uint32_t k = 0; k < I.num_geometries; ++k) gb.add(geom_box[I.first_geometry + k]);
        for (int corner = 0; corner < 8; ++corner) {
            const float p[3] = {(corner & 1) ? gb.hi[0] : gb.lo[0], (corner & 2) ? gb.hi[1] : gb.lo[1],
                                (corner & 4) ? gb.hi[2] : gb.lo[2]};
            float w[3];
            xform_point_h(M, p, w);
            world.add(w);
        }
        for (uint32_t k = 0; k < I.num_geometries; ++k) {
            const uint32_t g = I.first_geometry + k;
            const VptSurfaceGeometry& G = geoms[g];
            const uint32_t place = static_cast<uint32_t>(places.size());
            places.push_back(make_uint4(i, g, static_cast<uint32_t>(world_tris), 0u));
            world_tris += G.num_triangles;
            if (world_tris > kMaxTris) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: more than 2^28 world triangles");
            for (uint32_t t = 0; t < G.num_triangles; ++t) {
                if (prim_w[dgeom[g].prim_off + t] > 0 && inst_w[i] > 0) ++emitters;
                const uint32_t* ix = G.triangles + 3 * static_cast<size_t>(t);
                for (int v = 0; v < 3; ++v) {
                    float w[3];
                    xform_point_h(M, G.vertices + 9 * static_cast<size_t>(ix[v]), w);
                    tri_pos_f.insert(tri_pos_f.end(), w, w + 3);
                    float tag = 0.0f;
                    if (v == 0) std::memcpy(&tag, &place, sizeof(tag));
                    tri_pos.push_back(make_float4(w[0], w[1], w[2], tag));
                }
            }
        }
    }
    const float inst_integral = exclusive_cdf(inst_w.data(), ninst, inst_cdf.data());

    std::vector<BvhNode> nodes;
    std::vector<uint32_t> order;
    build_bvh(tri_pos_f, static_cast<uint32_t>(world_tris), &nodes, &order);

    Surfaces S{};
    int rc;
    if ((rc = upload(c, nodes, &S.nodes)) || (rc = upload(c, order, &S.order)) || (rc = upload(c, tri_pos, &S.tri_pos)) ||
        (rc = upload(c, places, &S.places)) || (rc = upload(c, dinst, &S.insts)) || (rc = upload(c, dgroup, &S.groups)) ||
        (rc = upload(c, dgeom, &S.geoms)) || (rc = upload(c, obj_tri, &S.obj_tri)) || (rc = upload(c, obj_nrm, &S.obj_nrm)) ||
        (rc = upload(c, obj_tan, &S.obj_tan)) || (rc = upload(c, dmat, &S.mats)) || (rc = upload(c, prim_w, &S.prim_w)) ||
        (rc = upload(c, prim_cdf, &S.prim_cdf)) || (rc = upload(c, group_w, &S.group_w)) ||
        (rc = upload(c, group_cdf, &S.group_cdf)) || (rc = upload(c, inst_w, &S.inst_w)) ||
        (rc = upload(c, inst_cdf, &S.inst_cdf))) {
        c->release_surfaces();
        return rc;
    }
    S.num_insts = ninst;
    S.num_tris = static_cast<uint32_t>(world_tris);
    S.inst_integral = inst_integral;
    S.enabled = 1;
    c->surf = new Surfaces(S);
    c->surf_nodes = static_cast<uint32_t>(nodes.size());
    c->surf_emitters = emitters;
    for (int a = 0; a < 3; ++a) {
        c->surf_box_min[a] = world.lo[a];
        c->surf_box_max[a] = world.hi[a];
    }
    c->update_world_box();
    return VPT_OK;
}

}  // namespace

void VptContextImpl::release_surfaces() {
    for (void* p : surf_mem) cudaFree(p);
    surf_mem.clear();
    delete surf;
    surf = nullptr;
    surf_nodes = surf_emitters = 0;
}

// finalizeWorldDimInfo (compute_light_probs.cu:139-157): the union of the instances' boxes and
// the volume's box; centre = midpoint, radius = |max - centre|.
void VptContextImpl::update_world_box() {
    bool any = false;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (has_volume) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = bbox_min[a];
            hi[a] = bbox_max[a];
        }
        any = true;
    }
    if (surf) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = any ? std::min(lo[a], surf_box_min[a]) : surf_box_min[a];
            hi[a] = any ? std::max(hi[a], surf_box_max[a]) : surf_box_max[a];
        }
        any = true;
    }
    float r2 = 0;
    for (int a = 0; a < 3; ++a) {
        world_min[a] = lo[a];
        world_max[a] = hi[a];
        const float center = (lo[a] + hi[a]) * 0.5f;
        const float d = hi[a] - center;
        r2 += d * d;
    }
    world_radius = any ? std::sqrt(r2) : 1.0f;
}

}  // namespace vpt

extern "C" {

int vpt_set_surfaces(VptContext* c, const VptSurfaceMaterial* materials, uint32_t num_materials,
                     const VptSurfaceGeometry* geometries, uint32_t num_geometries, const VptSurfaceInstance* instances,
                     uint32_t num_instances) {
    if (!c) return vpt::fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_surfaces: null context");
    try {
        return vpt::set_surfaces(c, materials, num_materials, geometries, num_geometries, instances, num_instances);
    } catch (const std::bad_alloc&) {
        c->release_surfaces();
        return vpt::fail(VPT_ERR_OUT_OF_MEMORY, "vpt_set_surfaces: host allocation failed");
    } catch (const std::exception& e) {
        c->release_surfaces();
        return vpt::fail(VPT_ERR_INVALID_ARGUMENT, std::string("vpt_set_surfaces: ") + e.what());
    }
}

int vpt_get_surface_info(VptContext* c, uint32_t* triangles, uint32_t* bvh_nodes, uint32_t* emitters, float* world_box) {
    if (!c) return vpt::fail(VPT_ERR_INVALID_ARGUMENT, "vpt_get_surface_info: null context");
    if (triangles) *triangles = c->surf ? c->surf->num_tris : 0;
    if (bvh_nodes) *bvh_nodes = c->surf_nodes;
    if (emitters) *emitters = c->surf_emitters;
    if (world_box) {
        for (int a = 0; a < 3; ++a) {
            world_box[a] = c->world_min[a];
            world_box[3 + a] = c->world_max[a];
        }
    }
    return VPT_OK;
}

int vpt_clear_volume(VptContext* c) {
    if (!c) return vpt::fail(VPT_ERR_INVALID_ARGUMENT, "vpt_clear_volume: null context");
    c->has_volume = false;
    c->update_world_box();
    return VPT_OK;
}

}  // extern "C"
