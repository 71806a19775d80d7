// Known-answer generator built against the reference's vendored NanoVDB 32.3 headers
// (ext/nanovdb/nanovdb, compiled by oracle/build_ref.sh into oracle/_ref/). Builds a small
// dense grid with the reference's GridBuilder and prints JSON with:
//   - the voxel values it was built from (x-major),
//   - the world bbox the renderer clips against (renderer_scene.cpp:494, 517-519),
//   - the global majorant of the renderer's scan over [min, max) (renderer_scene.cpp:498-509),
//   - first-order SampleFromVoxels results at index-space points,
//   - worldToIndexF results, and Ray::clip results against the float bbox.
#include <cstdio>
#include <random>
#include <vector>

#include <nanovdb/NanoVDB.h>
#include <nanovdb/util/GridBuilder.h>
#include <nanovdb/util/Ray.h>
#include <nanovdb/util/SampleFromVoxels.h>

static void pf(const char* name, const std::vector<float>& v, bool last = false) {
    std::printf("\"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.9g", i ? ", " : "", v[i]);
    std::printf("]%s\n", last ? "" : ",");
}

int main() {
    const int N = 20;
    const double dx = 1.0 / 16.0;
    const nanovdb::Vec3d origin(-0.625, -0.5, -0.375);
    std::mt19937 gen(777);
    std::uniform_real_distribution<float> u01(0.0f, 1.0f);
    std::vector<float> vox(N * N * N);
    nanovdb::GridBuilder<float> builder(0.0f);
    auto acc = builder.getAccessor();
    for (int x = 0; x < N; ++x)
        for (int y = 0; y < N; ++y)
            for (int z = 0; z < N; ++z) {
                float v = u01(gen);
                if (v < 0.2f) v = 0.0f;
                vox[(x * N + y) * N + z] = v;
                acc.setValue(nanovdb::Coord(x, y, z), v);
            }
    auto handle = builder.getHandle<>(dx, origin, "kat");
    const nanovdb::FloatGrid* grid = handle.grid<float>();
    auto wb = grid->worldBBox();
    auto ib = grid->indexBBox();
    const auto& racc = grid->tree().getAccessor();
    float majorant = -INFINITY;
    for (int ix = ib.min()[0]; ix < ib.max()[0]; ++ix)
        for (int iy = ib.min()[1]; iy < ib.max()[1]; ++iy)
            for (int iz = ib.min()[2]; iz < ib.max()[2]; ++iz) majorant = std::max(majorant, racc.getValue({ix, iy, iz}));

    // As in optix_pathtracing_kernels.cu:102-103: the sampler keeps a reference to the accessor.
    const nanovdb::DefaultReadAccessor<float>& sacc = grid->getAccessor();
    auto sampler = nanovdb::createSampler<1, nanovdb::DefaultReadAccessor<float>, false>(sacc);
    std::uniform_real_distribution<float> upos(-1.5f, N + 0.5f);
    std::vector<float> pts, vals;
    for (int i = 0; i < 512; ++i) {
        nanovdb::Vec3f p(upos(gen), upos(gen), upos(gen));
        if (i < 8) p = nanovdb::Vec3f(float(i), 7.0f + 0.25f * i, 8.0f - 0.5f * i);  // leaf-boundary cases
        pts.insert(pts.end(), {p[0], p[1], p[2]});
        vals.push_back(sampler(p));
    }
    std::uniform_real_distribution<float> uw(-1.0f, 1.0f);
    std::vector<float> wpts, widx;
    for (int i = 0; i < 128; ++i) {
        nanovdb::Vec3f p(uw(gen), uw(gen), uw(gen));
        nanovdb::Vec3f q = grid->worldToIndexF(p);
        wpts.insert(wpts.end(), {p[0], p[1], p[2]});
        widx.insert(widx.end(), {q[0], q[1], q[2]});
    }
    nanovdb::BBox<nanovdb::Vec3f> fbox(nanovdb::Vec3f(float(wb.min()[0]), float(wb.min()[1]), float(wb.min()[2])),
                                       nanovdb::Vec3f(float(wb.max()[0]), float(wb.max()[1]), float(wb.max()[2])));
    std::vector<float> rorg, rdir, rt;
    for (int i = 0; i < 256; ++i) {
        nanovdb::Vec3f o(3 * uw(gen), 3 * uw(gen), 3 * uw(gen));
        if (i % 4 == 0) o = nanovdb::Vec3f(0.5f * uw(gen), 0.5f * uw(gen), 0.5f * uw(gen));  // inside the box
        nanovdb::Vec3f d(uw(gen), uw(gen), uw(gen));
        if (i == 1) d = nanovdb::Vec3f(0.0f, 0.0f, 1.0f);
        if (i == 2) d = nanovdb::Vec3f(0.0f, -1.0f, 0.0f);
        d.normalize();
        nanovdb::Ray<float> ray(o, d, 0.0f, 1e10f);
        bool hit = ray.clip(fbox);
        rorg.insert(rorg.end(), {o[0], o[1], o[2]});
        rdir.insert(rdir.end(), {d[0], d[1], d[2]});
        rt.insert(rt.end(), {hit ? 1.0f : 0.0f, hit ? ray.t0() : 0.0f, hit ? ray.t1() : 0.0f});
    }
    std::printf("{\n\"n\": %d,\n\"voxel_size\": %.17g,\n\"origin\": [%.17g, %.17g, %.17g],\n", N, dx, origin[0], origin[1],
                origin[2]);
    std::printf("\"world_bbox\": [%.9g, %.9g, %.9g, %.9g, %.9g, %.9g],\n", float(wb.min()[0]), float(wb.min()[1]),
                float(wb.min()[2]), float(wb.max()[0]), float(wb.max()[1]), float(wb.max()[2]));
    std::printf("\"index_bbox\": [%d, %d, %d, %d, %d, %d],\n", ib.min()[0], ib.min()[1], ib.min()[2], ib.max()[0],
                ib.max()[1], ib.max()[2]);
    std::printf("\"global_majorant\": %.9g,\n", majorant);
    pf("voxels", vox);
    pf("sample_points", pts);
    pf("sample_values", vals);
    pf("world_points", wpts);
    pf("world_to_index", widx);
    pf("ray_origins", rorg);
    pf("ray_dirs", rdir);
    pf("ray_hit_t0_t1", rt, true);
    std::printf("}\n");
    return 0;
}
