// Fixture generator built against the reference's vendored NanoVDB 32.3 headers
// (ext/nanovdb/nanovdb, compiled by oracle/build_ref.sh into oracle/_ref/). Writes .nvdb files
// with the reference's own GridBuilder and io::writeGrid(s) into the directory argv[1], then
// prints JSON describing every grid as the reference reads it back (io::readGrid and the
// grid's own accessors):
//   - the file metadata (io::readGridMetaData) and the grid's map, world/index boxes, node
//     and tile counts, background;
//   - the global majorant of the renderer's scan over [min, max) of the index box
//     (renderer_scene.cpp:498-509) and the float clip box (renderer_scene.cpp:517-519);
//   - getValue at sample coordinates, an order-independent checksum of getValue over the
//     index box grown by two voxels, and first-order SampleFromVoxels values at points.
// Files written:
//   multi.nvdb       three grids, Codec::NONE: "density" (float, negative index coordinates,
//                    constant 8^3 blocks pruned to lower-node tiles), "block" (float, a constant
//                    128^3 region pruned to an upper-node tile) and "temperature" (double);
//   sphere_fog.nvdb  the reference's fog-volume sphere primitive (createFogVolumeSphere), whose
//                    interior is stored as tiles;
//   sphere_zip.nvdb  the same sphere written with Codec::ZIP.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include <nanovdb/NanoVDB.h>
#include <nanovdb/util/GridBuilder.h>
#include <nanovdb/util/IO.h>
#include <nanovdb/util/Primitives.h>
#include <nanovdb/util/SampleFromVoxels.h>

using nanovdb::Coord;
using nanovdb::CoordBBox;

// Order-independent, position-sensitive checksum of a voxel value: the same formula is
// evaluated by the tests on decoded leaves.
static uint64_t voxel_hash(int x, int y, int z, float v) {
    uint32_t bits;
    std::memcpy(&bits, &v, 4);
    uint64_t key = (uint64_t(uint32_t(x)) * 73856093ull) ^ (uint64_t(uint32_t(y)) * 19349663ull) ^
                   (uint64_t(uint32_t(z)) * 83492791ull);
    return (key | 1ull) * (uint64_t(bits) + 0x9E3779B97F4A7C15ull);
}

static float value_fn(const Coord& c, uint32_t seed) {
    // Smooth blob times a hashed speckle; about a third of the voxels are background.
    uint32_t h = uint32_t(c[0]) * 0x85EBCA77u ^ uint32_t(c[1]) * 0xC2B2AE3Du ^ uint32_t(c[2]) * 0x27D4EB2Fu ^ seed;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    float u = float(h >> 8) * (1.0f / 16777216.0f);
    float r2 = float(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    float blob = std::exp(-r2 / 180.0f);
    return u < 0.3f ? 0.0f : blob * (0.5f + u);
}

static void print_grid(const nanovdb::io::GridMetaData& meta, const nanovdb::GridHandle<nanovdb::HostBuffer>& h,
                       std::mt19937& gen, bool last) {
    std::printf("{\"name\": \"%s\", \"grid_type\": %u, \"grid_class\": %u, \"codec\": %u, \"grid_size\": %llu, ",
                meta.gridName.c_str(), unsigned(meta.gridType), unsigned(meta.gridClass), unsigned(meta.codec),
                (unsigned long long)meta.gridSize);
    std::printf("\"file_size\": %llu, \"voxel_count\": %llu, \"node_count\": [%u, %u, %u, %u], \"tile_count\": [%u, %u, %u], ",
                (unsigned long long)meta.fileSize, (unsigned long long)meta.voxelCount, meta.nodeCount[0],
                meta.nodeCount[1], meta.nodeCount[2], meta.nodeCount[3], meta.tileCount[0], meta.tileCount[1],
                meta.tileCount[2]);
    std::printf("\"meta_index_bbox\": [%d, %d, %d, %d, %d, %d], ", meta.indexBBox.min()[0], meta.indexBBox.min()[1],
                meta.indexBBox.min()[2], meta.indexBBox.max()[0], meta.indexBBox.max()[1], meta.indexBBox.max()[2]);
    std::printf("\"meta_world_bbox\": [%.17g, %.17g, %.17g, %.17g, %.17g, %.17g], ", meta.worldBBox.min()[0],
                meta.worldBBox.min()[1], meta.worldBBox.min()[2], meta.worldBBox.max()[0], meta.worldBBox.max()[1],
                meta.worldBBox.max()[2]);
    std::printf("\"meta_voxel_size\": [%.17g, %.17g, %.17g]", meta.voxelSize[0], meta.voxelSize[1], meta.voxelSize[2]);
    const nanovdb::FloatGrid* grid = h.grid<float>();
    if (!grid) {
        std::printf("}%s\n", last ? "" : ",");
        return;
    }
    auto wb = grid->worldBBox();
    auto ib = grid->indexBBox();
    const auto& map = grid->map();
    std::printf(", \"map_vec_d\": [%.17g, %.17g, %.17g], \"map_vec_f\": [%.9g, %.9g, %.9g], ", map.mVecD[0], map.mVecD[1],
                map.mVecD[2], map.mVecF[0], map.mVecF[1], map.mVecF[2]);
    std::printf("\"map_mat_f_diag\": [%.9g, %.9g, %.9g], \"map_inv_mat_f_diag\": [%.9g, %.9g, %.9g], ", map.mMatF[0],
                map.mMatF[4], map.mMatF[8], map.mInvMatF[0], map.mInvMatF[4], map.mInvMatF[8]);
    std::printf("\"background\": %.9g, ", grid->tree().background());
    // renderer_scene.cpp:517-519: the clip box is the double world box converted to float.
    std::printf("\"clip_box_f\": [%.9g, %.9g, %.9g, %.9g, %.9g, %.9g], ", float(wb.min()[0]), float(wb.min()[1]),
                float(wb.min()[2]), float(wb.max()[0]), float(wb.max()[1]), float(wb.max()[2]));
    std::printf("\"index_bbox\": [%d, %d, %d, %d, %d, %d], ", ib.min()[0], ib.min()[1], ib.min()[2], ib.max()[0],
                ib.max()[1], ib.max()[2]);
    const auto& acc = grid->tree().getAccessor();
    float majorant = -INFINITY;
    for (int ix = ib.min()[0]; ix < ib.max()[0]; ++ix)
        for (int iy = ib.min()[1]; iy < ib.max()[1]; ++iy)
            for (int iz = ib.min()[2]; iz < ib.max()[2]; ++iz) majorant = std::max(majorant, acc.getValue({ix, iy, iz}));
    std::printf("\"global_majorant\": %.9g, ", majorant);
    uint64_t sum_hash = 0, nonzero = 0;
    for (int ix = ib.min()[0] - 2; ix <= ib.max()[0] + 2; ++ix)
        for (int iy = ib.min()[1] - 2; iy <= ib.max()[1] + 2; ++iy)
            for (int iz = ib.min()[2] - 2; iz <= ib.max()[2] + 2; ++iz) {
                float v = acc.getValue({ix, iy, iz});
                sum_hash += voxel_hash(ix, iy, iz, v);
                nonzero += v != 0.0f;
            }
    std::printf("\"checksum_box\": [%d, %d, %d, %d, %d, %d], \"checksum\": \"%llu\", \"nonzero\": %llu, ",
                ib.min()[0] - 2, ib.min()[1] - 2, ib.min()[2] - 2, ib.max()[0] + 2, ib.max()[1] + 2, ib.max()[2] + 2,
                (unsigned long long)sum_hash, (unsigned long long)nonzero);
    std::uniform_int_distribution<int> ux(ib.min()[0] - 3, ib.max()[0] + 3), uy(ib.min()[1] - 3, ib.max()[1] + 3),
        uz(ib.min()[2] - 3, ib.max()[2] + 3);
    std::printf("\"coords\": [");
    std::vector<float> vals;
    for (int i = 0; i < 1024; ++i) {
        Coord c(ux(gen), uy(gen), uz(gen));
        std::printf("%s%d, %d, %d", i ? ", " : "", c[0], c[1], c[2]);
        vals.push_back(acc.getValue(c));
    }
    std::printf("], \"values\": [");
    for (size_t i = 0; i < vals.size(); ++i) std::printf("%s%.9g", i ? ", " : "", vals[i]);
    std::printf("], ");
    const nanovdb::DefaultReadAccessor<float>& sacc = grid->getAccessor();
    auto sampler = nanovdb::createSampler<1, nanovdb::DefaultReadAccessor<float>, false>(sacc);
    std::uniform_real_distribution<float> fx(ib.min()[0] - 1.5f, ib.max()[0] + 1.5f),
        fy(ib.min()[1] - 1.5f, ib.max()[1] + 1.5f), fz(ib.min()[2] - 1.5f, ib.max()[2] + 1.5f);
    std::printf("\"sample_points\": [");
    vals.clear();
    for (int i = 0; i < 256; ++i) {
        nanovdb::Vec3f p(fx(gen), fy(gen), fz(gen));
        std::printf("%s%.9g, %.9g, %.9g", i ? ", " : "", p[0], p[1], p[2]);
        vals.push_back(sampler(p));
    }
    std::printf("], \"sample_values\": [");
    for (size_t i = 0; i < vals.size(); ++i) std::printf("%s%.9g", i ? ", " : "", vals[i]);
    std::printf("]}%s\n", last ? "" : ",");
}

static void print_file(const std::string& label, const std::string& path, std::mt19937& gen, bool last) {
    auto metas = nanovdb::io::readGridMetaData(path);
    std::printf("\"%s\": [\n", label.c_str());
    for (size_t i = 0; i < metas.size(); ++i) {
        auto h = nanovdb::io::readGrid<nanovdb::HostBuffer>(path, uint64_t(i));
        print_grid(metas[i], h, gen, i + 1 == metas.size());
    }
    std::printf("]%s\n", last ? "" : ",");
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <output directory>\n", argv[0]);
        return 2;
    }
    const std::string dir = argv[1];
    std::vector<nanovdb::GridHandle<nanovdb::HostBuffer>> handles;
    {
        nanovdb::GridBuilder<float> b(0.0f, nanovdb::GridClass::FogVolume);
        // Constant 0.75 over [0,15]x[8,23]x[-16,-1]: eight whole leaves pruned to lower-node tiles.
        b([](const Coord& c) -> float {
              if (c[0] >= 0 && c[0] < 16 && c[1] >= 8 && c[1] < 24 && c[2] >= -16 && c[2] < 0) return 0.75f;
              return value_fn(c, 17u);
          },
          CoordBBox(Coord(-12, -9, -17), Coord(15, 23, 11)));
        handles.push_back(b.getHandle<>(0.0625, nanovdb::Vec3d(-0.25, 0.125, 0.5), "density"));
    }
    {
        nanovdb::GridBuilder<float> b(0.0f, nanovdb::GridClass::FogVolume);
        // x >= 128: a whole lower node of constant 0.5, pruned to an upper-node tile.
        b([](const Coord& c) -> float { return c[0] >= 128 ? 0.5f : value_fn(c, 99u); },
          CoordBBox(Coord(120, 0, 0), Coord(255, 127, 127)));
        handles.push_back(b.getHandle<>(0.01, nanovdb::Vec3d(-1.0, -0.5, -0.75), "block"));
    }
    {
        nanovdb::GridBuilder<double> b(0.0);
        b([](const Coord& c) -> double { return 1.0 + c[0] + 0.5 * c[1]; }, CoordBBox(Coord(0, 0, 0), Coord(9, 9, 9)));
        handles.push_back(b.getHandle<>(0.5, nanovdb::Vec3d(0.0), "temperature"));
    }
    nanovdb::io::writeGrids<nanovdb::HostBuffer, std::vector>(dir + "/multi.nvdb", handles);
    auto sphere = nanovdb::createFogVolumeSphere<float>(1.6f, nanovdb::Vec3f(0.3f, -0.2f, 0.5f), 0.1, 3.0,
                                                        nanovdb::Vec3d(0.05, -0.1, 0.2), "sphere_fog");
    nanovdb::io::writeGrid(dir + "/sphere_fog.nvdb", sphere);
    nanovdb::io::writeGrid(dir + "/sphere_zip.nvdb", sphere, nanovdb::io::Codec::ZIP);

    std::mt19937 gen(4242);
    std::printf("{\n");
    print_file("multi.nvdb", dir + "/multi.nvdb", gen, false);
    print_file("sphere_fog.nvdb", dir + "/sphere_fog.nvdb", gen, false);
    print_file("sphere_zip.nvdb", dir + "/sphere_zip.nvdb", gen, true);
    std::printf("}\n");
    return 0;
}
