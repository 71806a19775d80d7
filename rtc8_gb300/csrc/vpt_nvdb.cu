// NanoVDB grids as density volumes: a reader of the NanoVDB 32.x file format and in-memory grid
// layout (host code), and the sparse upload that turns a grid's leaves and tiles into the
// tracer's leaf table, leaf pool and majorant cells on the device.
//
// Replaces nanovdb::io::readGrid (ext/nanovdb/nanovdb/util/IO.h:576-606, called at
// renderer/renderer_scene.cpp:2468) followed by Scene::allocateVolumeGrid
// (renderer/renderer_scene.cpp:491-537). The reference uploads the NanoVDB buffer as it is and
// walks the tree on every lookup; here the tree is walked once on the host and flattened into
// 8^3 leaves behind a dense table, the layout every tracer kernel reads.
//
// Layout facts used below (NanoVDB.h, version 32: GridData :2185-2205, TreeData :2501-2507,
// RootData :2687-2747, InternalData :3043-3067, LeafData :3355-3372, io::Header/MetaData
// IO.h:112-158):
//   grid buffer:  GridData (672 B) | TreeData (64 B) | ... nodes, offsets relative to TreeData
//   root:         64 B header (index box, table size, background, stats) + 32-B tiles
//                 {u64 key, i64 child offset from the root, u32 state, value}
//   upper node:   32^3 children of 128^3 voxels, 270,400 B, child mask at 4128, table at 8256
//   lower node:   16^3 children of 8^3 voxels, 33,856 B, child mask at 544, table at 1088
//   leaf:         8^3 float values at byte 96, 2,144 B, origin = first 12 bytes & ~7
//   table entry:  8 B union of a tile value and a child offset relative to the node
//   file:         per segment a 16-B header {magic, version, grid count, codec}, one 176-B
//                 metadata record + name per grid, then the grids' payloads in order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "../../include/rtc8_vpt.h"
#include "vpt_ctx.h"
#include "vpt_scene.cuh"

namespace {

constexpr uint64_t kMagic = 0x304244566f6e614eULL;  // "NanoVDB0", little endian
constexpr uint32_t kMajorVersion = 32;
constexpr uint32_t kGridTypeFloat = 1;

constexpr uint64_t kGridDataBytes = 672;
constexpr uint64_t kTreeDataBytes = 64;
constexpr uint64_t kRootHeaderBytes = 64, kRootTileBytes = 32;
constexpr uint64_t kUpperBytes = 270400, kUpperChildMask = 4128, kUpperTable = 8256;
constexpr uint64_t kLowerBytes = 33856, kLowerChildMask = 544, kLowerTable = 1088;
constexpr uint64_t kLeafBytes = 2144, kLeafValues = 96;
constexpr uint64_t kFileHeaderBytes = 16, kMetaBytes = 176;

int fail(int code, const std::string& msg) { return vpt::ctx_set_error(code, msg.c_str()); }

// Bounds-checked little-endian reads from a byte span.
struct Span {
    const uint8_t* p;
    uint64_t n;
    bool has(uint64_t off, uint64_t len) const { return off <= n && len <= n - off; }
    template <typename T>
    T at(uint64_t off) const {
        T v;
        std::memcpy(&v, p + off, sizeof(T));
        return v;
    }
};

struct Region {  // a constant-valued cube of side `dim` voxels (a tile of the tree)
    int32_t origin[3];
    int32_t dim;
    float value;
};

struct Parsed {
    VptNanoVdbInfo info{};
    std::vector<uint64_t> leaf_offsets;  // byte offset of each leaf in the grid buffer
    std::vector<Region> tiles;           // tiles with a non-zero value
    std::vector<Region> root_regions;    // 4096^3 regions the root covers (child or tile)
};

int32_t key_coord(uint64_t key, int shift) {
    // RootData::KeyToCoord with USE_SINGLE_ROOT_KEY: 21-bit fields of (coord >> 12), the coordinate
    // rebuilt in 32-bit two's complement.
    return static_cast<int32_t>(static_cast<uint32_t>(((key >> shift) & ((1u << 21) - 1)) << 12));
}

bool mask_bit(const Span& s, uint64_t mask_off, uint32_t n) {
    uint64_t word = s.at<uint64_t>(mask_off + 8ull * (n >> 6));
    return (word >> (n & 63)) & 1u;
}

int parse_grid(const void* data, uint64_t bytes, Parsed* out) {
    if (!data) return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: null buffer");
    Span s{static_cast<const uint8_t*>(data), bytes};
    if (!s.has(0, kGridDataBytes + kTreeDataBytes)) return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: buffer too small");
    if (s.at<uint64_t>(0) != kMagic) return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: bad magic number");
    const uint32_t version = s.at<uint32_t>(16);
    if (((version >> 21) & 2047u) != kMajorVersion)
        return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: major version " + std::to_string((version >> 21) & 2047u) +
                                                  " (this reader handles 32)");
    VptNanoVdbInfo& info = out->info;
    const uint64_t grid_size = s.at<uint64_t>(32);
    if (grid_size > bytes) return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: buffer shorter than the grid size");
    info.grid_bytes = grid_size;
    std::memcpy(info.name, s.p + 40, 256);
    info.name[255] = 0;
    info.grid_class = s.at<uint32_t>(632);
    info.grid_type = s.at<uint32_t>(636);
    for (int a = 0; a < 3; ++a) {
        info.world_min[a] = s.at<double>(560 + 8 * a);
        info.world_max[a] = s.at<double>(584 + 8 * a);
        info.voxel_size[a] = s.at<double>(608 + 8 * a);
    }
    // Map (GridData + 296): matF[9], invMatF[9], vecF[3], taperF, matD[9], invMatD[9], vecD[3], taperD.
    const uint64_t map = 296;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            info.map_mat_f[3 * r + c] = s.at<float>(map + 4 * (3 * r + c));
            info.map_inv_mat_f[3 * r + c] = s.at<float>(map + 36 + 4 * (3 * r + c));
            info.map_mat_d[3 * r + c] = s.at<double>(map + 88 + 8 * (3 * r + c));
        }
    for (int a = 0; a < 3; ++a) {
        info.map_vec_f[a] = s.at<float>(map + 72 + 4 * a);
        info.map_vec_d[a] = s.at<double>(map + 232 + 8 * a);
    }
    const uint64_t tree = kGridDataBytes;
    uint64_t node_off[4];
    for (int l = 0; l < 4; ++l) node_off[l] = s.at<uint64_t>(tree + 8 * l);
    for (int l = 0; l < 3; ++l) {
        info.node_count[l] = s.at<uint32_t>(tree + 32 + 4 * l);
        info.tile_count[l] = s.at<uint32_t>(tree + 44 + 4 * l);
    }
    info.active_voxels = s.at<uint64_t>(tree + 56);
    if (info.grid_type != kGridTypeFloat) return VPT_OK;  // metadata only; the caller rejects non-float grids

    const uint64_t root = tree + node_off[3];
    if (!s.has(root, kRootHeaderBytes)) return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: root node out of range");
    for (int a = 0; a < 3; ++a) {
        info.index_min[a] = s.at<int32_t>(root + 4 * a);
        info.index_max[a] = s.at<int32_t>(root + 12 + 4 * a);
    }
    const uint32_t table_size = s.at<uint32_t>(root + 24);
    info.background = s.at<float>(root + 28);
    if (!s.has(root + kRootHeaderBytes, static_cast<uint64_t>(table_size) * kRootTileBytes))
        return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: root table out of range");

    // Walk root -> upper -> lower -> leaf. Child offsets must point forward inside the buffer and
    // the node counts must match the tree header, so a corrupt file cannot loop or read past it.
    uint64_t seen[3] = {0, 0, 0};
    for (uint32_t t = 0; t < table_size; ++t) {
        const uint64_t tile = root + kRootHeaderBytes + static_cast<uint64_t>(t) * kRootTileBytes;
        const uint64_t key = s.at<uint64_t>(tile);
        const int64_t child = s.at<int64_t>(tile + 8);
        const float value = s.at<float>(tile + 20);
        const int32_t uo[3] = {key_coord(key, 42), key_coord(key, 21), key_coord(key, 0)};
        out->root_regions.push_back({{uo[0], uo[1], uo[2]}, 4096, value});
        if (child == 0) {
            if (value != 0.0f) out->tiles.push_back({{uo[0], uo[1], uo[2]}, 4096, value});
            continue;
        }
        const uint64_t upper = root + static_cast<uint64_t>(child);
        if (child < 0 || !s.has(upper, kUpperBytes) || ++seen[2] > info.node_count[2])
            return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: bad upper-node reference");
        for (uint32_t n = 0; n < 32768u; ++n) {
            const int32_t lo[3] = {uo[0] + static_cast<int32_t>(((n >> 10) & 31u) << 7),
                                   uo[1] + static_cast<int32_t>(((n >> 5) & 31u) << 7),
                                   uo[2] + static_cast<int32_t>((n & 31u) << 7)};
            const uint64_t entry = upper + kUpperTable + 8ull * n;
            if (!mask_bit(s, upper + kUpperChildMask, n)) {
                const float v = s.at<float>(entry);
                if (v != 0.0f) out->tiles.push_back({{lo[0], lo[1], lo[2]}, 128, v});
                continue;
            }
            const int64_t lchild = s.at<int64_t>(entry);
            const uint64_t lower = upper + static_cast<uint64_t>(lchild);
            if (lchild <= 0 || !s.has(lower, kLowerBytes) || ++seen[1] > info.node_count[1])
                return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: bad lower-node reference");
            for (uint32_t m = 0; m < 4096u; ++m) {
                const int32_t fo[3] = {lo[0] + static_cast<int32_t>(((m >> 8) & 15u) << 3),
                                       lo[1] + static_cast<int32_t>(((m >> 4) & 15u) << 3),
                                       lo[2] + static_cast<int32_t>((m & 15u) << 3)};
                const uint64_t lentry = lower + kLowerTable + 8ull * m;
                if (!mask_bit(s, lower + kLowerChildMask, m)) {
                    const float v = s.at<float>(lentry);
                    if (v != 0.0f) out->tiles.push_back({{fo[0], fo[1], fo[2]}, 8, v});
                    continue;
                }
                const int64_t fchild = s.at<int64_t>(lentry);
                const uint64_t leaf = lower + static_cast<uint64_t>(fchild);
                if (fchild <= 0 || !s.has(leaf, kLeafBytes) || ++seen[0] > info.node_count[0])
                    return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: bad leaf reference");
                for (int a = 0; a < 3; ++a)
                    if ((s.at<int32_t>(leaf + 4 * a) & ~7) != fo[a])
                        return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: leaf origin does not match its position");
                out->leaf_offsets.push_back(leaf);
            }
        }
    }
    if (seen[0] != info.node_count[0] || seen[1] != info.node_count[1] || seen[2] != info.node_count[2])
        return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: node counts differ from the tree header");
    return VPT_OK;
}

// The box of voxels a lookup inside the grid's clip box can read: the clip box is the world
// image of [index_min, index_max + 1], and the first-order stencil of a point there reaches
// from floor(x) >= index_min - 1 to floor(x) + 1 <= index_max + 2; one more voxel of margin on
// each side absorbs rounding. Leaf-aligned, it becomes the extent of the tracer's leaf table.
void sample_extent(const VptNanoVdbInfo& info, int32_t lo[3], int32_t hi[3]) {
    for (int a = 0; a < 3; ++a) {
        lo[a] = (info.index_min[a] - 2) & ~7;
        hi[a] = ((info.index_max[a] + 2) & ~7) + 8;  // exclusive
    }
}

// Non-float grids, empty grids and maps that are not a uniform scale + translation are rejected.
int check_renderable(const VptNanoVdbInfo& info) {
    if (info.grid_type != kGridTypeFloat)
        return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid '" + std::string(info.name) + "' has grid type " +
                                                  std::to_string(info.grid_type) + "; density volumes must be float (1)");
    for (int a = 0; a < 3; ++a)
        if (info.index_min[a] > info.index_max[a])
            return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid '" + std::string(info.name) + "' has no active values");
    const float* m = info.map_mat_f;
    if (m[1] != 0 || m[2] != 0 || m[3] != 0 || m[5] != 0 || m[6] != 0 || m[7] != 0 || m[0] != m[4] || m[0] != m[8] ||
        !(m[0] > 0))
        return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid '" + std::string(info.name) +
                                                  "': only uniformly scaled, axis-aligned index-to-world maps are supported");
    for (int a = 0; a < 3; ++a)
        if (static_cast<int64_t>(info.index_max[a]) - info.index_min[a] > (1 << 20))
            return fail(VPT_ERR_INVALID_ARGUMENT, "NanoVDB grid: index box wider than 2^20 voxels");
    return VPT_OK;
}

// Flattens the grid into leaves covering the sample extent: the file's leaves inside it, then
// one constant leaf per 8^3 cell of every non-zero tile inside it, then (for a non-zero
// background) one background leaf per cell that no root entry covers. `origins` (3 per leaf)
// and `values` (512 per leaf, x<<6 | y<<3 | z) are filled when non-null; returns the count.
template <typename LeafFn>
int64_t flatten(const Span& s, const Parsed& g, LeafFn&& emit) {
    int32_t lo[3], hi[3];
    sample_extent(g.info, lo, hi);
    auto inside = [&](const int32_t o[3]) {
        return o[0] >= lo[0] && o[0] < hi[0] && o[1] >= lo[1] && o[1] < hi[1] && o[2] >= lo[2] && o[2] < hi[2];
    };
    int64_t count = 0;
    for (uint64_t leaf : g.leaf_offsets) {
        int32_t o[3];
        for (int a = 0; a < 3; ++a) o[a] = s.at<int32_t>(leaf + 4 * a) & ~7;
        if (!inside(o)) continue;
        emit(count++, o, reinterpret_cast<const float*>(s.p + leaf + kLeafValues), 0.0f);
    }
    auto fill_region = [&](const Region& r, float value) {
        int32_t a0[3], a1[3];
        for (int a = 0; a < 3; ++a) {
            a0[a] = std::max(r.origin[a], lo[a]);
            a1[a] = std::min(static_cast<int64_t>(r.origin[a]) + r.dim, static_cast<int64_t>(hi[a]));
        }
        for (int32_t x = a0[0]; x < a1[0]; x += 8)
            for (int32_t y = a0[1]; y < a1[1]; y += 8)
                for (int32_t z = a0[2]; z < a1[2]; z += 8) {
                    const int32_t o[3] = {x, y, z};
                    emit(count++, o, nullptr, value);
                }
    };
    for (const Region& r : g.tiles) fill_region(r, r.value);
    if (g.info.background != 0.0f) {
        for (int32_t x = lo[0] & ~4095; x < hi[0]; x += 4096)
            for (int32_t y = lo[1] & ~4095; y < hi[1]; y += 4096)
                for (int32_t z = lo[2] & ~4095; z < hi[2]; z += 4096) {
                    bool covered = false;
                    for (const Region& r : g.root_regions)
                        covered |= r.origin[0] == x && r.origin[1] == y && r.origin[2] == z;
                    if (!covered) fill_region({{x, y, z}, 4096, g.info.background}, g.info.background);
                }
    }
    return count;
}

// Scans the segments of an .nvdb file (io::Segment::read, IO.h:481-509) for the grid with
// running index `grid_index` and fills its metadata record (MetaData, IO.h:144-158) and the
// absolute byte offset of its payload. The payloads of a segment follow its header and all
// of its metadata records, in grid order.
int parse_file_header(FILE* f, uint64_t grid_index, VptNanoVdbInfo* info) {
    uint64_t counter = 0, pos = 0;
    bool found = false;
    for (;;) {
        uint8_t hdr[kFileHeaderBytes];
        const size_t got = std::fread(hdr, 1, sizeof(hdr), f);
        if (got == 0) break;
        if (got != sizeof(hdr)) return fail(VPT_ERR_INVALID_ARGUMENT, "nvdb file: truncated segment header");
        pos += sizeof(hdr);
        Span h{hdr, sizeof(hdr)};
        const uint64_t magic = h.at<uint64_t>(0);
        if (magic != kMagic) {
            if (__builtin_bswap64(magic) == kMagic)
                return fail(VPT_ERR_INVALID_ARGUMENT, "nvdb file: reversed endianness");
            return fail(VPT_ERR_INVALID_ARGUMENT, "nvdb file: bad magic number (not a NanoVDB file)");
        }
        const uint32_t version = h.at<uint32_t>(8);
        if (((version >> 21) & 2047u) != kMajorVersion)
            return fail(VPT_ERR_INVALID_ARGUMENT, "nvdb file: major version " + std::to_string((version >> 21) & 2047u) +
                                                      " (this reader handles 32)");
        const uint16_t grid_count = h.at<uint16_t>(12);
        const uint16_t codec = h.at<uint16_t>(14);
        uint64_t before = 0, segment_payload = 0;  // payload bytes before the wanted grid, in total
        bool here = false;
        for (uint16_t g = 0; g < grid_count; ++g, ++counter) {
            uint8_t meta[kMetaBytes];
            if (std::fread(meta, 1, sizeof(meta), f) != sizeof(meta))
                return fail(VPT_ERR_INVALID_ARGUMENT, "nvdb file: truncated grid metadata");
            pos += sizeof(meta);
            Span m{meta, sizeof(meta)};
            const uint32_t name_size = m.at<uint32_t>(136);
            if (name_size > (1u << 20)) return fail(VPT_ERR_INVALID_ARGUMENT, "nvdb file: bad grid-name size");
            std::string name(name_size, '\0');
            if (name_size && std::fread(&name[0], 1, name_size, f) != name_size)
                return fail(VPT_ERR_INVALID_ARGUMENT, "nvdb file: truncated grid name");
            pos += name_size;
            const uint64_t file_bytes = m.at<uint64_t>(8);
            if (counter == grid_index) {
                found = here = true;
                before = segment_payload;
                *info = VptNanoVdbInfo{};
                std::snprintf(info->name, sizeof(info->name), "%s", name.c_str());
                info->grid_bytes = m.at<uint64_t>(0);
                info->file_bytes = file_bytes;
                info->active_voxels = m.at<uint64_t>(24);
                info->grid_type = m.at<uint32_t>(32);
                info->grid_class = m.at<uint32_t>(36);
                for (int a = 0; a < 3; ++a) {
                    info->world_min[a] = m.at<double>(40 + 8 * a);
                    info->world_max[a] = m.at<double>(64 + 8 * a);
                    info->index_min[a] = m.at<int32_t>(88 + 4 * a);
                    info->index_max[a] = m.at<int32_t>(100 + 4 * a);
                    info->voxel_size[a] = m.at<double>(112 + 8 * a);
                }
                for (int l = 0; l < 3; ++l) {
                    info->node_count[l] = m.at<uint32_t>(140 + 4 * l);
                    info->tile_count[l] = m.at<uint32_t>(156 + 4 * l);
                }
                info->codec = codec;
            }
            segment_payload += file_bytes;
        }
        if (here) info->payload_offset = pos + before;
        if (std::fseek(f, static_cast<long>(segment_payload), SEEK_CUR) != 0)
            return fail(VPT_ERR_INVALID_ARGUMENT, "nvdb file: truncated grid payload");
        pos += segment_payload;
    }
    if (!found)
        return fail(VPT_ERR_INVALID_ARGUMENT, "nvdb file: grid index " + std::to_string(grid_index) +
                                                  " exceeds the grid count " + std::to_string(counter));
    info->grid_count = static_cast<uint32_t>(counter);
    return VPT_OK;
}

// Host memory the flattened grid may take: at most 2^26 leaves (128 GiB of values, more than one
// GPU holds) over at most 2^30 leaf cells (4 GiB of table).
constexpr int64_t kMaxFlatLeaves = int64_t(1) << 26;
constexpr int64_t kMaxLeafCells = int64_t(1) << 30;

// Runs an ABI body so that no C++ exception crosses the C boundary: host allocation failures
// become VPT_ERR_OUT_OF_MEMORY, anything else VPT_ERR_INVALID_ARGUMENT.
template <class F>
int guarded(const char* what, F&& body) {
    try {
        return body();
    } catch (const std::bad_alloc&) {
        return fail(VPT_ERR_OUT_OF_MEMORY, std::string(what) + ": out of host memory");
    } catch (const std::exception& e) {
        return fail(VPT_ERR_INVALID_ARGUMENT, std::string(what) + ": " + e.what());
    } catch (...) {
        return fail(VPT_ERR_INVALID_ARGUMENT, std::string(what) + ": unexpected error");
    }
}

}  // namespace

extern "C" {

int vpt_nvdb_file_info(const char* path, uint64_t grid_index, VptNanoVdbInfo* info) {
    if (!path || !info) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_nvdb_file_info: bad arguments");
    return guarded("vpt_nvdb_file_info", [&] {
        FILE* f = std::fopen(path, "rb");
        if (!f) return fail(VPT_ERR_INVALID_ARGUMENT, std::string("vpt_nvdb_file_info: cannot open ") + path);
        int rc = parse_file_header(f, grid_index, info);
        std::fclose(f);
        return rc;
    });
}

int vpt_nanovdb_grid_info(const void* grid, uint64_t bytes, VptNanoVdbInfo* info) {
    return guarded("vpt_nanovdb_grid_info", [&] {
    if (!info) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_nanovdb_grid_info: null info");
    Parsed g;
    int rc = parse_grid(grid, bytes, &g);
    if (rc) return rc;
    *info = g.info;
    if (g.info.grid_type == kGridTypeFloat) {
        sample_extent(g.info, info->extent_min, info->extent_max);
        Span s{static_cast<const uint8_t*>(grid), bytes};
        info->flat_leaves = flatten(s, g, [](int64_t, const int32_t*, const float*, float) {});
    }
    return VPT_OK;
    });
}

int vpt_nanovdb_decode_leaves(const void* grid, uint64_t bytes, int64_t capacity, int32_t* leaf_origins,
                              float* leaf_values, int64_t* count) {
    return guarded("vpt_nanovdb_decode_leaves", [&] {
    if (!count) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_nanovdb_decode_leaves: null count");
    Parsed g;
    int rc = parse_grid(grid, bytes, &g);
    if (rc) return rc;
    if ((rc = check_renderable(g.info))) return rc;
    Span s{static_cast<const uint8_t*>(grid), bytes};
    const int64_t n = flatten(s, g, [](int64_t, const int32_t*, const float*, float) {});
    *count = n;
    if (!leaf_origins && !leaf_values) return VPT_OK;
    if (capacity < n)
        return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_nanovdb_decode_leaves: capacity " + std::to_string(capacity) +
                                                  " < " + std::to_string(n) + " leaves");
    flatten(s, g, [&](int64_t i, const int32_t* o, const float* vals, float constant) {
        if (leaf_origins)
            for (int a = 0; a < 3; ++a) leaf_origins[3 * i + a] = o[a];
        if (leaf_values) {
            float* dst = leaf_values + 512 * i;
            if (vals)
                std::memcpy(dst, vals, 512 * sizeof(float));
            else
                std::fill(dst, dst + 512, constant);
        }
    });
    return VPT_OK;
    });
}

int vpt_set_volume_nanovdb(VptContext* c, const void* grid, uint64_t bytes) {
    return guarded("vpt_set_volume_nanovdb", [&] {
    if (!c) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_volume_nanovdb: null context");
    Parsed g;
    int rc = parse_grid(grid, bytes, &g);
    if (rc) return rc;
    if ((rc = check_renderable(g.info))) return rc;
    int32_t lo[3], hi[3];
    sample_extent(g.info, lo, hi);
    const int32_t lx = (hi[0] - lo[0]) / 8, ly = (hi[1] - lo[1]) / 8, lz = (hi[2] - lo[2]) / 8;
    const int64_t cells = static_cast<int64_t>(lx) * ly * lz;
    if (cells > kMaxLeafCells)
        return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_volume_nanovdb: grid too large (" + std::to_string(cells) +
                                                  " leaf cells, at most 2^30)");
    Span s{static_cast<const uint8_t*>(grid), bytes};
    const int64_t n = flatten(s, g, [](int64_t, const int32_t*, const float*, float) {});
    if (n > kMaxFlatLeaves)
        return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_volume_nanovdb: grid too large (" + std::to_string(n) +
                                                  " leaves, at most 2^26)");
    std::vector<int32_t> table(static_cast<size_t>(cells), -1);
    std::vector<int32_t> origins(static_cast<size_t>(3 * n));
    std::vector<float> values(static_cast<size_t>(512 * std::max<int64_t>(n, 1)));
    bool dup = false;
    flatten(s, g, [&](int64_t i, const int32_t* o, const float* vals, float constant) {
        const int64_t cell = ((static_cast<int64_t>(o[0] - lo[0]) / 8) * ly + (o[1] - lo[1]) / 8) * lz + (o[2] - lo[2]) / 8;
        dup |= table[cell] >= 0;
        table[cell] = static_cast<int32_t>(i);
        for (int a = 0; a < 3; ++a) origins[3 * i + a] = o[a] - lo[a];
        float* dst = values.data() + 512 * i;
        if (vals)
            std::memcpy(dst, vals, 512 * sizeof(float));
        else
            std::fill(dst, dst + 512, constant);
    });
    if (dup) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_volume_nanovdb: two nodes cover the same 8^3 cell");
    return vpt::upload_sparse_grid(c, table, lx, ly, lz, origins, values.data(), n, lo, g.info);
    });
}

int vpt_set_volume_nvdb_file(VptContext* c, const char* path, uint64_t grid_index) {
    return guarded("vpt_set_volume_nvdb_file", [&] {
    if (!c || !path) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_volume_nvdb_file: bad arguments");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(VPT_ERR_INVALID_ARGUMENT, std::string("vpt_set_volume_nvdb_file: cannot open ") + path);
    VptNanoVdbInfo info{};
    int rc = parse_file_header(f, grid_index, &info);
    if (rc) {
        std::fclose(f);
        return rc;
    }
    if (info.codec != 0) {
        std::fclose(f);
        return fail(VPT_ERR_INVALID_ARGUMENT,
                    std::string("vpt_set_volume_nvdb_file: grid '") + info.name + "' is stored with codec " +
                        std::to_string(info.codec) +
                        " (1 = ZIP, 2 = BLOSC); decompress it on the host and pass the grid to vpt_set_volume_nanovdb");
    }
    std::vector<uint8_t> buf(static_cast<size_t>(info.grid_bytes));
    const bool ok = std::fseek(f, static_cast<long>(info.payload_offset), SEEK_SET) == 0 &&
                    std::fread(buf.data(), 1, buf.size(), f) == buf.size();
    std::fclose(f);
    if (!ok) return fail(VPT_ERR_INVALID_ARGUMENT, "vpt_set_volume_nvdb_file: truncated grid payload");
    return vpt_set_volume_nanovdb(c, buf.data(), buf.size());
    });
}

}  // extern "C"
