// Scene set-up kernels: procedural fBm density volumes, the sparse 8^3-leaf grid with its
// majorant cells, and the environment importance map.
#include "vpt_scene.cuh"

#include <cfloat>

namespace vpt {
namespace {

// ------------------------------------------------------------------------------ fBm volume
__device__ __forceinline__ uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

// Lattice hash of the value noise: integer mixing only, so host and device agree exactly.
__device__ __forceinline__ float lattice_value(int ix, int iy, int iz, uint32_t seed) {
    uint32_t h = seed * 0x9E3779B1u;
    h ^= static_cast<uint32_t>(ix) * 0x85EBCA77u;
    h = rotl32(h, 13) * 0xC2B2AE3Du;
    h ^= static_cast<uint32_t>(iy) * 0x85EBCA77u;
    h = rotl32(h, 13) * 0xC2B2AE3Du;
    h ^= static_cast<uint32_t>(iz) * 0x85EBCA77u;
    h = rotl32(h, 13) * 0xC2B2AE3Du;
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    h *= 0x846ca68bu;
    h ^= h >> 16;
    return static_cast<float>(h >> 8) * (1.0f / 16777216.0f);
}

__device__ __forceinline__ float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }

__device__ float value_noise(float x, float y, float z, uint32_t seed) {
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    int ix = static_cast<int>(fx), iy = static_cast<int>(fy), iz = static_cast<int>(fz);
    float wx = fade(x - fx), wy = fade(y - fy), wz = fade(z - fz);
    float c[2][2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int d = 0; d < 2; ++d) c[a][b][d] = lattice_value(ix + a, iy + b, iz + d, seed);
    auto lerp = [](float a, float b, float w) { return a + w * (b - a); };
    float x00 = lerp(c[0][0][0], c[1][0][0], wx);
    float x10 = lerp(c[0][1][0], c[1][1][0], wx);
    float x01 = lerp(c[0][0][1], c[1][0][1], wx);
    float x11 = lerp(c[0][1][1], c[1][1][1], wx);
    float y0 = lerp(x00, x10, wy);
    float y1 = lerp(x01, x11, wy);
    return lerp(y0, y1, wz);
}

__global__ void fbm_kernel(float* __restrict__ out, int n, uint32_t seed, int octaves, float lacunarity, float gain,
                           float base_frequency) {
    int64_t total = static_cast<int64_t>(n) * n * n;
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < total;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int z = static_cast<int>(idx % n);
        int y = static_cast<int>((idx / n) % n);
        int x = static_cast<int>(idx / (static_cast<int64_t>(n) * n));
        float px = (x + 0.5f) / n, py = (y + 0.5f) / n, pz = (z + 0.5f) / n;
        float freq = base_frequency, amp = 1.0f, sum = 0.0f, norm = 0.0f;
        for (int o = 0; o < octaves; ++o) {
            sum += amp * value_noise(px * freq, py * freq, pz * freq, seed + 1013u * static_cast<uint32_t>(o));
            norm += amp;
            amp *= gain;
            freq *= lacunarity;
        }
        out[idx] = sum / norm;
    }
}

__global__ void minmax_kernel(const float* __restrict__ v, int64_t n, unsigned int* __restrict__ mm) {
    float lo = FLT_MAX, hi = 0.0f;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float x = v[i];
        lo = fminf(lo, x);
        hi = fmaxf(hi, x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        // Values are non-negative: their IEEE bit patterns order like unsigned integers.
        atomicMin(mm, __float_as_uint(lo));
        atomicMax(mm + 1, __float_as_uint(hi));
    }
}

__global__ void remap_kernel(float* __restrict__ v, int64_t n, const unsigned int* __restrict__ mm, float threshold) {
    float lo = __uint_as_float(mm[0]), hi = __uint_as_float(mm[1]);
    float scale = hi > lo ? 1.0f / (hi - lo) : 0.0f;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float r = (v[i] - lo) * scale;
        if (threshold > 0.0f) r = r > threshold ? (r - threshold) / (1.0f - threshold) : 0.0f;
        v[i] = r;
    }
}

__global__ void max_into_kernel(float* __restrict__ a, const float* __restrict__ b, int64_t n) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        a[i] = fmaxf(a[i], b[i]);
}

// ------------------------------------------------------------------------------ sparse grid
// One CTA per leaf cell: activity (any non-zero voxel), and the cell majorant = max over the
// cell's voxels with a one-voxel apron below and a two-voxel apron above (the trilinear
// stencil of a point in the cell reaches one voxel past it), so the majorant bounds every
// sample taken inside the cell, including points a rounding error outside it.
__global__ void leaf_stats_kernel(const float* __restrict__ dense, int nx, int ny, int nz, int lx, int ly, int lz,
                                  int32_t* __restrict__ active, float* __restrict__ cell_maj) {
    int64_t cell = blockIdx.x;
    int cz = static_cast<int>(cell % lz);
    int cy = static_cast<int>((cell / lz) % ly);
    int cx = static_cast<int>(cell / (static_cast<int64_t>(lz) * ly));
    float any = 0.0f, mx = 0.0f;
    for (int q = threadIdx.x; q < 11 * 11 * 11; q += blockDim.x) {
        int dz = q % 11, dy = (q / 11) % 11, dx = q / 121;
        int x = cx * 8 - 1 + dx, y = cy * 8 - 1 + dy, z = cz * 8 - 1 + dz;
        if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) continue;
        float v = dense[(static_cast<int64_t>(x) * ny + y) * nz + z];
        mx = fmaxf(mx, v);
        if (dx >= 1 && dx <= 8 && dy >= 1 && dy <= 8 && dz >= 1 && dz <= 8 && v != 0.0f) any = 1.0f;
    }
    __shared__ float s_mx[32], s_any[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        any = fmaxf(any, __shfl_xor_sync(0xffffffffu, any, o));
    }
    if ((threadIdx.x & 31) == 0) {
        s_mx[threadIdx.x >> 5] = mx;
        s_any[threadIdx.x >> 5] = any;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.0f, a = 0.0f;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
            m = fmaxf(m, s_mx[w]);
            a = fmaxf(a, s_any[w]);
        }
        cell_maj[cell] = m;
        active[cell] = a > 0.0f ? 1 : 0;
    }
}

__global__ void pack_leaves_kernel(const float* __restrict__ dense, int nx, int ny, int nz, int lx, int ly, int lz,
                                   const int32_t* __restrict__ table, float* __restrict__ values) {
    int64_t cell = blockIdx.x;
    int32_t slot = table[cell];
    if (slot < 0) return;
    int cz = static_cast<int>(cell % lz);
    int cy = static_cast<int>((cell / lz) % ly);
    int cx = static_cast<int>(cell / (static_cast<int64_t>(lz) * ly));
    for (int q = threadIdx.x; q < 512; q += blockDim.x) {
        int x = cx * 8 + (q >> 6), y = cy * 8 + ((q >> 3) & 7), z = cz * 8 + (q & 7);
        float v = 0.0f;
        if (x < nx && y < ny && z < nz) v = dense[(static_cast<int64_t>(x) * ny + y) * nz + z];
        values[static_cast<int64_t>(slot) * 512 + q] = v;
    }
}

// leaf_stats_kernel for a grid held as leaves behind a table (absent leaves read 0): a cell
// whose 3x3x3 neighbourhood of cells holds no leaf gets majorant 0 without reading voxels.
__global__ void sparse_leaf_stats_kernel(const int32_t* __restrict__ table, const float* __restrict__ values, int lx,
                                         int ly, int lz, float* __restrict__ cell_maj) {
    const int64_t cell = blockIdx.x;
    const int cz = static_cast<int>(cell % lz);
    const int cy = static_cast<int>((cell / lz) % ly);
    const int cx = static_cast<int>(cell / (static_cast<int64_t>(lz) * ly));
    __shared__ int s_near;
    __shared__ float s_mx[32];
    if (threadIdx.x == 0) s_near = 0;
    __syncthreads();
    if (threadIdx.x < 27) {
        const int x = cx + static_cast<int>(threadIdx.x / 9) - 1, y = cy + static_cast<int>((threadIdx.x / 3) % 3) - 1,
                  z = cz + static_cast<int>(threadIdx.x % 3) - 1;
        if (x >= 0 && y >= 0 && z >= 0 && x < lx && y < ly && z < lz &&
            table[(static_cast<int64_t>(x) * ly + y) * lz + z] >= 0)
            s_near = 1;
    }
    __syncthreads();
    if (!s_near) {
        if (threadIdx.x == 0) cell_maj[cell] = 0.0f;
        return;
    }
    const int nx = 8 * lx, ny = 8 * ly, nz = 8 * lz;
    float mx = 0.0f;
    for (int q = threadIdx.x; q < 11 * 11 * 11; q += blockDim.x) {
        const int dz = q % 11, dy = (q / 11) % 11, dx = q / 121;
        const int x = cx * 8 - 1 + dx, y = cy * 8 - 1 + dy, z = cz * 8 - 1 + dz;
        if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) continue;
        const int32_t slot = table[(static_cast<int64_t>(x >> 3) * ly + (y >> 3)) * lz + (z >> 3)];
        if (slot < 0) continue;
        mx = fmaxf(mx, values[static_cast<int64_t>(slot) * 512 + (((x & 7) << 6) | ((y & 7) << 3) | (z & 7))]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) s_mx[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.0f;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) m = fmaxf(m, s_mx[w]);
        cell_maj[cell] = m;
    }
}

// Maximum of the leaf voxels inside [lo, hi) (non-negative start, so the float bits order like
// unsigned integers).
__global__ void leaf_box_max_kernel(const float* __restrict__ values, const int32_t* __restrict__ origins,
                                    int64_t total, int3 lo, int3 hi, unsigned int* out) {
    float mx = 0.0f;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t slot = i >> 9;
        const int q = static_cast<int>(i & 511);
        const int x = origins[3 * slot] + (q >> 6), y = origins[3 * slot + 1] + ((q >> 3) & 7),
                  z = origins[3 * slot + 2] + (q & 7);
        if (x >= lo.x && x < hi.x && y >= lo.y && y < hi.y && z >= lo.z && z < hi.z) mx = fmaxf(mx, values[i]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(mx));
}

// renderer_scene.cpp:498-509: the reference scans index coordinates [min, max) of the
// inclusive index box, i.e. every voxel but the last plane along each axis.
__global__ void global_max_kernel(const float* __restrict__ dense, int nx, int ny, int nz, unsigned int* out) {
    int64_t total = static_cast<int64_t>(nx - 1) * (ny - 1) * (nz - 1);
    float mx = 0.0f;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int z = static_cast<int>(i % (nz - 1));
        int y = static_cast<int>((i / (nz - 1)) % (ny - 1));
        int x = static_cast<int>(i / (static_cast<int64_t>(nz - 1) * (ny - 1)));
        mx = fmaxf(mx, dense[(static_cast<int64_t>(x) * ny + y) * nz + z]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(mx));
}

// ------------------------------------------------------------------------------ importance map
// compute_light_probs.cu:161-184 (first mip: luminance * pi/2 * sin(theta) inside the image).
__global__ void imp_first_mip_kernel(const float4* __restrict__ env, int w, int h, int map_w, int map_h,
                                     float* __restrict__ mip0) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= map_w || y >= map_h) return;
    float importance = 0.0f;
    if (x < w && y < h) {
        float4 t = env[static_cast<int64_t>(y) * w + x];
        float correction = kPi / 2 * sinf(kPi * (y + 0.5f) / h);
        importance = (0.2126729f * t.x + 0.7151522f * t.y + 0.0721750f * t.z) * correction;
    }
    mip0[static_cast<int64_t>(y) * map_w + x] = importance;
}

// compute_light_probs.cu:186-211 (2x2 average; the last level also yields the integral).
__global__ void imp_mip_kernel(const float* __restrict__ src, int sw, int sh, float* __restrict__ dst, int dw, int dh,
                               int last, int num_mips, float* __restrict__ integral) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    int srow = max(sw, 1);
    float sum = 0.0f;
    if (2 * x < sw && 2 * y < sh) sum += src[static_cast<int64_t>(2 * y) * srow + 2 * x];
    if (2 * x + 1 < sw && 2 * y < sh) sum += src[static_cast<int64_t>(2 * y) * srow + 2 * x + 1];
    if (2 * x < sw && 2 * y + 1 < sh) sum += src[static_cast<int64_t>(2 * y + 1) * srow + 2 * x];
    if (2 * x + 1 < sw && 2 * y + 1 < sh) sum += src[static_cast<int64_t>(2 * y + 1) * srow + 2 * x + 1];
    sum *= 0.25f;
    dst[static_cast<int64_t>(y) * dw + x] = sum;
    if (last) *integral = sum * static_cast<float>(1u << (2 * (num_mips - 1)));
}

}  // namespace

void generate_fbm(float* dense, int n, uint32_t seed, int octaves, float lacunarity, float gain, float base_frequency,
                  float threshold, unsigned int* d_minmax, cudaStream_t s) {
    int64_t total = static_cast<int64_t>(n) * n * n;
    int blocks = static_cast<int>(std::min<int64_t>((total + 255) / 256, 152 * 32));
    fbm_kernel<<<blocks, 256, 0, s>>>(dense, n, seed, octaves, lacunarity, gain, base_frequency);
    unsigned int init[2] = {0x7f7fffffu, 0u};
    cudaMemcpyAsync(d_minmax, init, sizeof(init), cudaMemcpyHostToDevice, s);
    minmax_kernel<<<blocks, 256, 0, s>>>(dense, total, d_minmax);
    remap_kernel<<<blocks, 256, 0, s>>>(dense, total, d_minmax, threshold);
}

void max_into(float* a, const float* b, int64_t n, cudaStream_t s) {
    const int blocks = static_cast<int>(std::min<int64_t>((n + 255) / 256, 152 * 32));
    max_into_kernel<<<blocks, 256, 0, s>>>(a, b, n);
}

void leaf_stats(const float* dense, int nx, int ny, int nz, int lx, int ly, int lz, int32_t* active, float* cell_maj,
                cudaStream_t s) {
    int64_t cells = static_cast<int64_t>(lx) * ly * lz;
    leaf_stats_kernel<<<static_cast<unsigned int>(cells), 256, 0, s>>>(dense, nx, ny, nz, lx, ly, lz, active, cell_maj);
}

void pack_leaves(const float* dense, int nx, int ny, int nz, int lx, int ly, int lz, const int32_t* table,
                 float* values, cudaStream_t s) {
    int64_t cells = static_cast<int64_t>(lx) * ly * lz;
    pack_leaves_kernel<<<static_cast<unsigned int>(cells), 256, 0, s>>>(dense, nx, ny, nz, lx, ly, lz, table, values);
}

void sparse_leaf_stats(const int32_t* table, const float* values, int lx, int ly, int lz, float* cell_maj,
                       cudaStream_t s) {
    const int64_t cells = static_cast<int64_t>(lx) * ly * lz;
    if (cells > 0)
        sparse_leaf_stats_kernel<<<static_cast<unsigned int>(cells), 128, 0, s>>>(table, values, lx, ly, lz, cell_maj);
}

void leaf_box_max(const float* values, const int32_t* origins, int64_t slots, const int32_t box_lo[3],
                  const int32_t box_hi[3], unsigned int* out, cudaStream_t s) {
    cudaMemsetAsync(out, 0, sizeof(unsigned int), s);
    if (slots <= 0) return;
    const int64_t total = slots * 512;
    const int blocks = static_cast<int>(std::min<int64_t>((total + 255) / 256, 152 * 16));
    leaf_box_max_kernel<<<blocks, 256, 0, s>>>(values, origins, total, make_int3(box_lo[0], box_lo[1], box_lo[2]),
                                               make_int3(box_hi[0], box_hi[1], box_hi[2]), out);
}

void global_max(const float* dense, int nx, int ny, int nz, unsigned int* out, cudaStream_t s) {
    cudaMemsetAsync(out, 0, sizeof(unsigned int), s);
    if (nx < 2 || ny < 2 || nz < 2) return;
    global_max_kernel<<<152 * 8, 256, 0, s>>>(dense, nx, ny, nz, out);
}

void build_importance_map(const float4* env, int w, int h, int map_w, int map_h, int num_mips,
                          const int64_t* offsets, float* mips, float* d_integral, cudaStream_t s) {
    dim3 block(32, 8);
    dim3 grid0((map_w + 31) / 32, (map_h + 7) / 8);
    imp_first_mip_kernel<<<grid0, block, 0, s>>>(env, w, h, map_w, map_h, mips + offsets[0]);
    for (int l = 1; l < num_mips; ++l) {
        int sw = map_w >> (l - 1), sh = map_h >> (l - 1);
        int dw = std::max(map_w >> l, 1), dh = std::max(map_h >> l, 1);
        dim3 grid((dw + 31) / 32, (dh + 7) / 8);
        imp_mip_kernel<<<grid, block, 0, s>>>(mips + offsets[l - 1], sw, sh, mips + offsets[l], dw, dh,
                                              l == num_mips - 1, num_mips, d_integral);
    }
}

}  // namespace vpt
