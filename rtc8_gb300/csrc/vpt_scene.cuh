// Scene set-up kernels (procedural volume, sparse grid build, importance map).
#pragma once

#include "vpt_device.cuh"

#include <algorithm>

namespace vpt {

void generate_fbm(float* dense, int n, uint32_t seed, int octaves, float lacunarity, float gain, float base_frequency,
                  float threshold, unsigned int* d_minmax, cudaStream_t s);
// a[i] = max(a[i], b[i]) (union of two clouds).
void max_into(float* a, const float* b, int64_t n, cudaStream_t s);
void leaf_stats(const float* dense, int nx, int ny, int nz, int lx, int ly, int lz, int32_t* active, float* cell_maj,
                cudaStream_t s);
void pack_leaves(const float* dense, int nx, int ny, int nz, int lx, int ly, int lz, const int32_t* table,
                 float* values, cudaStream_t s);
// Sparse grid built from leaves (vpt_nvdb.cu): cell majorants with the apron of leaf_stats, read
// through the leaf table; and the maximum over the voxels of the leaves inside the index box
// [box_lo, box_hi) (extent-relative coordinates), as float bits in *out.
void sparse_leaf_stats(const int32_t* table, const float* values, int lx, int ly, int lz, float* cell_maj,
                       cudaStream_t s);
void leaf_box_max(const float* values, const int32_t* origins, int64_t slots, const int32_t box_lo[3],
                  const int32_t box_hi[3], unsigned int* out, cudaStream_t s);
void global_max(const float* dense, int nx, int ny, int nz, unsigned int* out, cudaStream_t s);
void build_importance_map(const float4* env, int w, int h, int map_w, int map_h, int num_mips,
                          const int64_t* offsets, float* mips, float* d_integral, cudaStream_t s);

}  // namespace vpt
