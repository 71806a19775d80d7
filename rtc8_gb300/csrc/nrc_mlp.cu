// Neural radiance cache: a fully fused FP16 MLP (64-wide hidden layers, ReLU, no biases) on the
// Blackwell tensor cores. Replaces tiny-cuda-nn's FullyFusedMLP + encodings + Trainer
// (renderer/network_interface.cu:50-192), including the reference's default position encoding,
// the multiresolution hash grid (network_interface.cu:99-122), whose tables are gathered into the
// first layer's operand tile, trained by a scatter-add of the first layer's input gradient, and
// updated by the same Adam / EMA kernel as the weights.
//
// One CTA of 128 threads works on 128-row tiles (one thread per row): the encoded input tile
// and every hidden activation tile are FP16 in shared memory (core-matrix layout, nrc_tc.cuh),
// the weights are copied once per CTA into shared memory in the same layout, and each layer is
// one chain of tcgen05.mma (M = 128, N = 64 or 16, K = 16 per instruction) into an FP32 TMEM
// accumulator, read back with tcgen05.ld for the ReLU / FP16 epilogue. Training keeps all
// activations of a tile on chip; the backward pass reads activations and weights transposed
// through MN-major descriptors (no transposed copies) and reduces weight gradients with FP32
// vector atomics. Adam (with L2 regularisation) and an optional EMA of the weights run in one
// elementwise kernel that also repacks the FP16 weight images.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/rtc8_nrc.h"
#include "nrc_tc.cuh"

namespace nrc {
namespace {

thread_local std::string g_err;
int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
#define NRC_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail(NRC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr int kTile = 128;
constexpr int kWidth = 64;
constexpr int kOutPad = 16;
constexpr int kMaxMats = 8;
constexpr float kPiF = 3.14159265358979323846f;

// Multiresolution hash grid of the reference's HashGrid option (network_interface.cu:99-109):
// 16 levels of 2 features, at most 2^15 entries per level, base resolution 16, per-level scale 2.
constexpr int kGridLevels = 16;
constexpr int kGridFeatures = 2;
constexpr uint32_t kGridMaxEntries = 1u << 15;
constexpr float kGridBaseResolution = 16.0f;
constexpr float kGridLog2PerLevelScale = 1.0f;  // log2(2)

// Network shape: matrix j maps in[j] -> out[j] features; matrix 0 reads the encoded input.
struct NetLayout {
    int enc;
    int in_dim;
    int in_real;           // encoded features before padding
    int L;                 // number of weight matrices (hidden layers + 1)
    int in[kMaxMats], out[kMaxMats];
    int poff[kMaxMats];    // FP32 parameter offset of matrix j
    uint32_t boff[kMaxMats];  // byte offset of matrix j in the FP16 weight image
    int nparams;           // MLP weights; hash-grid parameters follow them in the parameter vector
    uint32_t blob_bytes;
    int out_act;
    float loss_scale;
    // Hash grid (NRC_ENCODING_HASHGRID only): level l holds grid_size[l] entries of two features,
    // entries grid_off[l] .. grid_off[l] + grid_size[l] of the table image; a lattice point of the
    // level's grid_res^3 lattice is stored densely or hashed (bit l of grid_hashed).
    int grid_params;       // 2 x entries, 0 without the hash grid
    uint32_t grid_off[kGridLevels], grid_size[kGridLevels], grid_res[kGridLevels];
    float grid_scale[kGridLevels];
    uint32_t grid_hashed;
};

// Level geometry of the hash grid: scale 16 * 2^l - 1, resolution ceil(scale) + 1, table size
// min(resolution^3 rounded up to a multiple of 8, 2^15), hashed when the lattice outgrows it.
void grid_layout(NetLayout& l) {
    uint32_t off = 0;
    l.grid_hashed = 0;
    for (int lv = 0; lv < kGridLevels; ++lv) {
        const float scale = std::exp2(static_cast<float>(lv) * kGridLog2PerLevelScale) * kGridBaseResolution - 1.0f;
        const uint32_t res = static_cast<uint32_t>(std::ceil(scale)) + 1u;
        const uint64_t cells = static_cast<uint64_t>(res) * res * res;
        const uint64_t padded = (cells + 7) / 8 * 8;
        const uint32_t size = static_cast<uint32_t>(std::min<uint64_t>(padded, kGridMaxEntries));
        l.grid_scale[lv] = scale;
        l.grid_res[lv] = res;
        l.grid_size[lv] = size;
        l.grid_off[lv] = off;
        if (cells > size) l.grid_hashed |= 1u << lv;
        off += size;
    }
    l.grid_params = static_cast<int>(off) * kGridFeatures;
}

NetLayout make_layout(int enc, int hidden, int out_act, float loss_scale) {
    NetLayout l{};
    l.enc = enc;
    l.in_dim = enc == NRC_ENCODING_VOLUME ? 144 : 64;
    l.in_real = enc == NRC_ENCODING_VOLUME ? 138 : (enc == NRC_ENCODING_HASHGRID ? 58 : 62);
    if (enc == NRC_ENCODING_HASHGRID) grid_layout(l);
    l.L = hidden + 1;
    int po = 0;
    uint32_t bo = 0;
    for (int j = 0; j < l.L; ++j) {
        l.in[j] = j == 0 ? l.in_dim : kWidth;
        l.out[j] = j == l.L - 1 ? kOutPad : kWidth;
        l.poff[j] = po;
        l.boff[j] = bo;
        po += l.in[j] * l.out[j];
        bo += static_cast<uint32_t>(l.in[j] * l.out[j] * 2);
    }
    l.nparams = po;
    l.blob_bytes = bo;
    l.out_act = out_act;
    l.loss_scale = loss_scale;
    return l;
}

// ------------------------------------------------------------------------------ encodings
// The FP16 encoded input of one query goes into row `r` of a [128][K] core-matrix tile, eight
// features (one 16-byte store) at a time. Every feature index is a compile-time constant after
// unrolling, so the features stay in registers.
__device__ __forceinline__ void store8(uint8_t* tile, int r, int chunk, int K, const float (&v)[8]) {
    uint4 w;
    w.x = pack_half2(v[0], v[1]);
    w.y = pack_half2(v[2], v[3]);
    w.z = pack_half2(v[4], v[5]);
    w.w = pack_half2(v[6], v[7]);
    *reinterpret_cast<uint4*>(tile + cm_offset(r, chunk * 8, K)) = w;
}

__device__ __forceinline__ float one_blob(float x, int b, int nbins) {
    float z = (x - (b + 0.5f) / nbins) * nbins;
    return __expf(-0.5f * z * z);
}

// NRC_ENCODING_REFERENCE (64 features): TriangleWave(12) on the 3 position coordinates
// (feature 12a + f), OneBlob(4) on the 5 angle / roughness inputs, angles divided by pi or 2 pi
// (feature 36 + 4a + b), identity on the 6 reflectance values (56..61), 2 zeros.
__device__ __forceinline__ float reference_feature(int i, const float* q) {
    if (i < 36) {
        const float v = q[i / 12] * static_cast<float>(1 << (i % 12));
        const float fr = v - floorf(v);
        return 2.0f * fabsf(fr - 0.5f);
    }
    if (i < 56) {
        const int a = (i - 36) / 4, b = (i - 36) % 4;
        const float scale = a == 4 ? 1.0f : ((a & 1) ? 1.0f / 6.28318531f : 1.0f / 3.14159265f);
        return one_blob(q[3 + a] * scale, b, 4);
    }
    if (i < 62) return q[8 + (i - 56)];
    return 0.0f;
}

// Eight consecutive one-blob bins b0 .. b0 + 7 of x (already scaled by the bin count):
// g_b = exp(-z_b^2 / 2), z_b = x - (b + 0.5). From the exact value at bin b0 + 4, the neighbours
// follow by the ratios g_{b+1} / g_b = exp(z_b - 1/2) and g_{b-1} / g_b = exp(-z_b - 1/2), each
// ratio shrinking by e^-1 per step: three special-function evaluations for eight bins instead of
// eight (the relative error of the products stays near 1e-6, far below the FP16 rounding).
// For |z| up to the bin count no intermediate overflows; where the centre value underflows to 0
// every bin of the group is below e^-40 and encodes as 0 in FP16.
__device__ __forceinline__ void one_blob8(float x, int b0, float (&v)[8]) {
    constexpr float kInvE = 0.36787944117144233f;
    const float z = x - (static_cast<float>(b0 + 4) + 0.5f);
    const float g = __expf(-0.5f * z * z);
    float up = __expf(z - 0.5f);   // g_{c+1} / g_c
    float dn = __expf(-z - 0.5f);  // g_{c-1} / g_c
    v[4] = g;
    float gu = g, gd = g;
#pragma unroll
    for (int j = 1; j <= 3; ++j) {
        gu *= up;
        up *= kInvE;
        v[4 + j] = gu;
        gd *= dn;
        dn *= kInvE;
        v[4 - j] = gd;
    }
    gd *= dn;
    v[0] = gd;
}

// NRC_ENCODING_VOLUME (144 features): sin and cos of pi 2^f x for the 3 position coordinates
// (features 2(12a + f) and 2(12a + f) + 1), OneBlob(32) on vOut theta / pi and phi / 2 pi
// (feature 72 + 32a + b), the local density (roughness slot) and the albedo (diffuse.r), 6 zeros.
__device__ __forceinline__ void encode_row_volume(const float* q, uint8_t* tile, int r) {
    constexpr int K = 144;
    // Chunk k holds frequencies f0 .. f0 + 3 (f0 = 4 (k % 3)) of coordinate k / 3.
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        // sin / cos(pi v) with v = x 2^f0 exact: v = m + r (m integer, r in [0, 1)), so
        // sin(pi v) = (-1)^m sin(pi r) and likewise cos; the hardware approximation on [0, pi)
        // is accurate to ~4e-7. The next three frequencies follow by angle doubling,
        // sin 2a = 2 sin a cos a, cos 2a = (cos a - sin a)(cos a + sin a), which at most
        // multiplies that error by 8 (~3e-6, far below the FP16 rounding of the features).
        const float x = q[k / 3] * static_cast<float>(1 << (4 * (k % 3)));
        const float m = floorf(x);
        float sn, cs;
        __sincosf(kPiF * (x - m), &sn, &cs);
        const float sign = (static_cast<int>(m) & 1) ? -1.0f : 1.0f;
        sn *= sign;
        cs *= sign;
        float v[8];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            v[2 * i] = sn;
            v[2 * i + 1] = cs;
            const float s2 = 2.0f * sn * cs;
            cs = (cs - sn) * (cs + sn);
            sn = s2;
        }
        store8(tile, r, k, K, v);
    }
    const float theta = q[5] * (32.0f / 3.14159265f), phi = q[6] * (32.0f / 6.28318531f);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float v[8];
        one_blob8(k < 4 ? theta : phi, 8 * (k % 4), v);
        store8(tile, r, 9 + k, K, v);
    }
    const float last[8] = {q[7], q[8], 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    store8(tile, r, 17, K, last);
}

// The 8 lattice corners of a position in hash-grid level `lv`: table entries (feature pairs) and
// trilinear weights. pos = scale x + 1/2 (one rounding), corner c takes floor(pos) + bit d of c
// on axis d with weight frac or 1 - frac; dense levels index x + y res + z res^2, hashed levels
// x ^ 2654435761 y ^ 805459861 z (the published spatial hash of the multiresolution hash
// encoding, Mueller et al. 2022), both modulo the level's table size.
__device__ __forceinline__ void grid_corners(const NetLayout& ly, int lv, const float* p, uint32_t (&e)[8],
                                             float (&w)[8]) {
    const float scale = ly.grid_scale[lv];
    const uint32_t res = ly.grid_res[lv], size = ly.grid_size[lv], off = ly.grid_off[lv];
    const bool hashed = (ly.grid_hashed >> lv) & 1u;
    float fr[3];
    uint32_t g[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float pos = fmaf(scale, p[d], 0.5f);
        const float fl = floorf(pos);
        fr[d] = pos - fl;
        g[d] = static_cast<uint32_t>(static_cast<int>(fl));
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint32_t x = g[0] + (c & 1), y = g[1] + ((c >> 1) & 1), z = g[2] + ((c >> 2) & 1);
        const float wx = (c & 1) ? fr[0] : 1.0f - fr[0];
        const float wy = (c & 2) ? fr[1] : 1.0f - fr[1];
        const float wz = (c & 4) ? fr[2] : 1.0f - fr[2];
        w[c] = (wx * wy) * wz;
        const uint32_t i = hashed ? (x ^ (y * 2654435761u) ^ (z * 805459861u)) : (x + (y + z * res) * res);
        // i modulo the level's size without a division: a hashed level has 2^15 entries (a mask);
        // a dense level's corner indices stay below res^3 + res^2 + res < 2 size (one subtraction).
        e[c] = off + (hashed ? (i & (size - 1u)) : (i >= size ? i - size : i));
    }
}

// Hash-grid position in [0, 1]^3 (positions outside the world box are clamped to it).
__device__ __forceinline__ void grid_position(const float* q, float (&p)[3]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) p[d] = fminf(fmaxf(q[d], 0.0f), 1.0f);
}

// NRC_ENCODING_HASHGRID (64 features): levels 0..15 x 2 features from the FP16 tables (feature
// 2 lv + f), then the reference encoding's OneBlob(4) on the 5 angle / roughness inputs
// (32 + 4a + b) and identity on the 6 reflectance values (52..57), 6 zeros.
__device__ __forceinline__ void encode_row_hashgrid(const NetLayout& ly, const uint32_t* __restrict__ grid,
                                                    const float* q, uint8_t* tile, int r) {
    float p[3];
    grid_position(q, p);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float v[8];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            uint32_t e[8];
            float w[8];
            grid_corners(ly, 4 * k + h, p, e, w);
            uint32_t raw[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) raw[c] = __ldg(grid + e[c]);
            float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&raw[c]));
                f0 += w[c] * f.x;
                f1 += w[c] * f.y;
            }
            v[2 * h] = f0;
            v[2 * h + 1] = f1;
        }
        store8(tile, r, k, 64, v);
    }
#pragma unroll
    for (int k = 4; k < 8; ++k) {
        float v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] = reference_feature(8 * k + i + 4, q);
        store8(tile, r, k, 64, v);
    }
}

// Adds the gradient of the 32 hash-grid features of one query (`d`, loss-scaled) into the FP32
// table gradient: corner c of level lv receives w_c x d[2 lv + f].
__device__ __forceinline__ void grid_backward(const NetLayout& ly, const float* q, const float (&d)[32],
                                              float* __restrict__ grid_grad) {
    float p[3];
    grid_position(q, p);
#pragma unroll 1
    for (int lv = 0; lv < kGridLevels; ++lv) {
        const float d0 = d[2 * lv], d1 = d[2 * lv + 1];
        if (d0 == 0.0f && d1 == 0.0f) continue;
        uint32_t e[8];
        float w[8];
        grid_corners(ly, lv, p, e, w);
#pragma unroll
        for (int c = 0; c < 8; ++c)
            atomicAdd(reinterpret_cast<float2*>(grid_grad) + e[c], make_float2(w[c] * d0, w[c] * d1));
    }
}

// Kernels specialised for the 144-wide volume input compile only its encoder.
template <int IN>
__device__ __forceinline__ void encode_row(const NetLayout& ly, const uint32_t* __restrict__ grid, const float* q,
                                           uint8_t* tile, int r) {
    if constexpr (IN == 144) {
        encode_row_volume(q, tile, r);
    } else if (ly.enc == NRC_ENCODING_REFERENCE) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = reference_feature(8 * k + i, q);
            store8(tile, r, k, 64, v);
        }
    } else {
        encode_row_hashgrid(ly, grid, q, tile, r);
    }
}

// Record of row `row` of a launch: the row itself, or idx[row] for an indexed launch.
__device__ __forceinline__ uint32_t record_of(const uint32_t* __restrict__ idx, uint32_t row) {
    return idx ? __ldg(idx + row) : row;
}

__device__ __forceinline__ void load_query(const float* __restrict__ in, const uint32_t* __restrict__ idx, uint32_t row,
                                           uint32_t n, float* q) {
    if (row < n) {
        const float2* p = reinterpret_cast<const float2*>(in + static_cast<size_t>(record_of(idx, row)) * 14);
#pragma unroll
        for (int i = 0; i < 7; ++i) {
            float2 v = __ldg(p + i);
            q[2 * i] = v.x;
            q[2 * i + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < 14; ++i) q[i] = 0.0f;
    }
}

// ------------------------------------------------------------------------------ MMA helpers
// D (128 x N, TMEM) = A (128 x K, smem, K-major) * W^T where W is N x K (K-major). Step ks reads the
// operands 256 bytes further on (two core matrices along K), i.e. 16 more in the descriptors'
// start-address field; the known K of the networks' layers (144, 64) unroll, so one thread issues
// the chain without recomputing descriptors (measured: inference 0.618 -> 0.589 ms per 2^23
// queries, the single-thread issue of an N = 64 MMA then takes ~49 cycles, not ~62).
__device__ __forceinline__ void issue_layer(uint32_t tmem_d, uint32_t a_addr, uint32_t w_addr, int K, int N) {
    const uint32_t idesc = idesc_f16(kTile, N, 0, 0);
    const uint64_t ad = smem_desc(a_addr, 128, static_cast<uint32_t>(K * 16));
    const uint64_t bd = smem_desc(w_addr, 128, static_cast<uint32_t>(K * 16));
    if (K == 144) {
#pragma unroll
        for (int ks = 0; ks < 9; ++ks) mma_f16(tmem_d, ad + 16 * ks, bd + 16 * ks, idesc, ks > 0 ? 1u : 0u);
    } else if (K == 64) {
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) mma_f16(tmem_d, ad + 16 * ks, bd + 16 * ks, idesc, ks > 0 ? 1u : 0u);
    } else {
        for (int ks = 0; ks < K / 16; ++ks) mma_f16(tmem_d, ad + 16 * ks, bd + 16 * ks, idesc, ks > 0 ? 1u : 0u);
    }
}

// As issue_layer with A read from tensor memory: a_tmem holds the 128 x K FP16 activations
// (row = lane, K elements packed two per 32-bit column).
__device__ __forceinline__ void issue_layer_ts(uint32_t tmem_d, uint32_t a_tmem, uint32_t w_addr, int K, int N) {
    const uint32_t idesc = idesc_f16(kTile, N, 0, 0);
    const uint64_t bd = smem_desc(w_addr, 128, static_cast<uint32_t>(K * 16));
    if (K == 64) {
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) mma_f16_ts(tmem_d, a_tmem + ks * 8, bd + 16 * ks, idesc, ks > 0 ? 1u : 0u);
    } else {
        for (int ks = 0; ks < K / 16; ++ks) mma_f16_ts(tmem_d, a_tmem + ks * 8, bd + 16 * ks, idesc, ks > 0 ? 1u : 0u);
    }
}

// Writes 16 FP32 values (columns c0..c0+15 of row r) as FP16 into a [128][K] core-matrix tile.
__device__ __forceinline__ void store_row16(uint8_t* tile, int r, int c0, int K, const float (&v)[16]) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        uint4 w;
        w.x = pack_half2(v[8 * h + 0], v[8 * h + 1]);
        w.y = pack_half2(v[8 * h + 2], v[8 * h + 3]);
        w.z = pack_half2(v[8 * h + 4], v[8 * h + 5]);
        w.w = pack_half2(v[8 * h + 6], v[8 * h + 7]);
        *reinterpret_cast<uint4*>(tile + cm_offset(r, c0 + 8 * h, K)) = w;
    }
}
// As store_row16 with ReLU fused into the FP16 conversion.
__device__ __forceinline__ void store_row16_relu(uint8_t* tile, int r, int c0, int K, const float (&v)[16]) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        uint4 w;
        w.x = pack_half2_relu(v[8 * h + 0], v[8 * h + 1]);
        w.y = pack_half2_relu(v[8 * h + 2], v[8 * h + 3]);
        w.z = pack_half2_relu(v[8 * h + 4], v[8 * h + 5]);
        w.w = pack_half2_relu(v[8 * h + 6], v[8 * h + 7]);
        *reinterpret_cast<uint4*>(tile + cm_offset(r, c0 + 8 * h, K)) = w;
    }
}
// Reads 16 FP16 values (columns c0..c0+15 of row r) of a core-matrix tile.
__device__ __forceinline__ void load_row16(const uint8_t* tile, int r, int c0, int K, float (&v)[16]) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        uint4 w = *reinterpret_cast<const uint4*>(tile + cm_offset(r, c0 + 8 * h, K));
        const __half2* p = reinterpret_cast<const __half2*>(&w);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float2 f = __half22float2(p[i]);
            v[8 * h + 2 * i] = f.x;
            v[8 * h + 2 * i + 1] = f.y;
        }
    }
}

constexpr uint32_t kErrTimeout = 1u;

__host__ __device__ __forceinline__ uint32_t align_up(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }

// ------------------------------------------------------------------------------ inference
// G independent groups of 128 threads per CTA, each with its own 128-row tile, mbarrier and 64
// TMEM columns, share one copy of the weights in shared memory. The groups' per-layer chains
// (MMA, then the TMEM -> ReLU -> FP16 epilogue) are not synchronised with each other, so while
// one group runs its epilogue or encodes its next input, the tensor cores serve another: G tiles
// in flight per SM instead of one per CTA. A group reuses its input tile's shared memory for the
// hidden activations (a layer's MMA has completed before its epilogue overwrites the operand).
__host__ __device__ constexpr uint32_t infer_tile_bytes(int in_dim) { return (kTile * in_dim * 2 + 1023) / 1024 * 1024; }

// TA: the hidden activations stay in tensor memory (32 packed FP16 columns per group next to the
// group's 64 accumulator columns) and feed the next layer's MMA as its A operand; only the encoded
// input tile goes through shared memory.
// idx (optional): row r of the launch is record idx[r] of `in` and `out`.
template <int IN, int G, bool TA>
__global__ void __launch_bounds__(kTile* G, 1) mlp_infer_kernel(const NetLayout ly, const uint8_t* __restrict__ blob,
                                                             const uint32_t* __restrict__ grid,
                                                             const float* __restrict__ in,
                                                             const uint32_t* __restrict__ idx,
                                                             const uint32_t* __restrict__ dev_n, uint32_t n_max,
                                                             float* __restrict__ out, unsigned int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr uint32_t kTileBytes = infer_tile_bytes(IN);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int g = tid / kTile, gt = tid % kTile;  // group, row of the tile
    const uint32_t bar_id = 1 + g;                // named barrier of the group (0 = whole CTA)
    uint8_t* s_w = smem;
    uint8_t* s_t = smem + align_up(ly.blob_bytes, 1024) + g * kTileBytes;
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(smem + align_up(ly.blob_bytes, 1024) + G * kTileBytes);
    uint32_t* s_slot = reinterpret_cast<uint32_t*>(s_bar + G);

    for (uint32_t i = tid; i < ly.blob_bytes / 16; i += kTile * G)
        reinterpret_cast<uint4*>(s_w)[i] = __ldg(reinterpret_cast<const uint4*>(blob) + i);
    constexpr uint32_t kCols = TA ? 128 : 64;  // TMEM columns per group
    if (warp == 0) tmem_alloc(s_slot, kCols * G);
    if (gt == 0) {
        mbar_init(s_bar + g, 1);
        mbar_fence_init();
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *s_slot;
    const uint32_t tmem = tmem_base + kCols * g;                     // the group's accumulator columns
    const uint32_t tmem_a = tmem + 64;                               // TA: the group's activation columns
    const uint32_t lane_base = static_cast<uint32_t>((warp % 4) * 32) << 16;  // lanes = rows of the tile
    const uint32_t n = dev_n ? min(*dev_n, n_max) : n_max;
    const uint32_t ntiles = (n + kTile - 1) / kTile;
    uint32_t phase = 0;
    bool ok = true;
    float q[14];
    const uint32_t stride = gridDim.x * G;
    load_query(in, idx, (blockIdx.x * G + g) * kTile + gt, n, q);
    for (uint32_t tile = blockIdx.x * G + g; tile < ntiles && ok; tile += stride) {
        const uint32_t row = tile * kTile + gt;
        encode_row<IN>(ly, grid, q, s_t, gt);
        // The next tile's queries load while this tile runs through the layers. (Encoding it
        // during layer 1, when the input tile is already free in the TA form, measured slower:
        // the group's next epilogue waits for the encoder.)
        load_query(in, idx, (tile + stride) * kTile + gt, n, q);
        fence_async_smem();
        named_sync(bar_id, kTile);
        for (int j = 0; j < ly.L && ok; ++j) {
            if (gt == 0) {
                tc_fence_after();
                if (TA && j > 0)
                    issue_layer_ts(tmem, tmem_a, smem_u32(s_w + ly.boff[j]), ly.in[j], ly.out[j]);
                else
                    issue_layer(tmem, smem_u32(s_t), smem_u32(s_w + ly.boff[j]), ly.in[j], ly.out[j]);
                mma_commit(s_bar + g);
            }

            ok = named_sync_and(bar_id, kTile, mbar_wait(s_bar + g, phase));  // group-uniform decision
            phase ^= 1;
            tc_fence_after();
            if (!ok) break;
            if (j < ly.L - 1 && TA) {
                // ReLU + FP16 pack of the accumulator straight back into tensor memory.
#pragma unroll
                for (int c = 0; c < kWidth / 32; ++c) {
                    float v0[16], v1[16];
                    tmem_ld16(tmem + lane_base + c * 32, v0);
                    tmem_ld16(tmem + lane_base + c * 32 + 16, v1);
                    tmem_wait_ld();
                    uint32_t w[16];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        w[i] = pack_half2_relu(v0[2 * i], v0[2 * i + 1]);
                        w[8 + i] = pack_half2_relu(v1[2 * i], v1[2 * i + 1]);
                    }
                    tmem_st16(tmem_a + lane_base + c * 16, w);
                }
                tmem_wait_st();
                tc_fence_before();
                named_sync(bar_id, kTile);
            } else if (j < ly.L - 1) {
#pragma unroll
                for (int c = 0; c < kWidth / 32; ++c) {  // two TMEM loads in flight per wait
                    float v0[16], v1[16];
                    tmem_ld16(tmem + lane_base + c * 32, v0);
                    tmem_ld16(tmem + lane_base + c * 32 + 16, v1);
                    tmem_wait_ld();
                    store_row16_relu(s_t, gt, c * 32, kWidth, v0);
                    store_row16_relu(s_t, gt, c * 32 + 16, kWidth, v1);
                }
                tc_fence_before();
                fence_async_smem();
                named_sync(bar_id, kTile);
            } else {
                float v[16];
                tmem_ld16(tmem + lane_base, v);
                tmem_wait_ld();
                if (row < n) {
                    float* o = out + static_cast<size_t>(record_of(idx, row)) * 3;
#pragma unroll
                    for (int c = 0; c < 3; ++c) o[c] = ly.out_act == NRC_OUTPUT_EXP ? __expf(v[c]) : v[c];
                }
                tc_fence_before();
                named_sync(bar_id, kTile);
            }
        }
    }
    if (!ok && gt == 0) atomicOr(err, kErrTimeout);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem_base, kCols * G);
}

// ------------------------------------------------------------------------------ training
// One CTA per 128-sample tile: forward keeping all activations, relative-L2-luminance loss
// gradient (denominator held constant), backward with weight gradients reduced into `grad`
// (scaled by loss_scale) and the batch loss added to `loss`.
// With the hash grid the backward pass also computes the first layer's input gradient and
// scatters its 32 hash features into the table gradient (grad + ly.nparams).
template <int IN>
__global__ void __launch_bounds__(kTile) mlp_train_kernel(const NetLayout ly, const uint8_t* __restrict__ blob,
                                                          const uint32_t* __restrict__ grid,
                                                          const float* __restrict__ in, const float* __restrict__ target,
                                                          uint32_t n, float* __restrict__ grad, float* __restrict__ loss,
                                                          unsigned int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int L = ly.L;
    uint8_t* s_w = smem;
    uint8_t* s_act0 = smem + align_up(ly.blob_bytes, 1024);
    uint8_t* s_acts = s_act0 + kTile * IN * 2;             // act_1 .. act_{L-1}, 16 KB each
    uint8_t* s_dza = s_acts + (L - 1) * kTile * kWidth * 2;
    uint8_t* s_dzb = s_dza + kTile * kWidth * 2;
    uint8_t* s_dzo = s_dzb + kTile * kWidth * 2;            // output gradient tile, 128 x 16
    uint8_t* s_slack = s_dzo + kTile * kOutPad * 2;         // absorbs MN-major over-reads
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_slack + 2048);
    uint32_t* s_slot = reinterpret_cast<uint32_t*>(s_bar + 1);
    auto act = [&](int j) -> uint8_t* { return j == 0 ? s_act0 : s_acts + (j - 1) * kTile * kWidth * 2; };

    for (uint32_t i = tid; i < ly.blob_bytes / 16; i += kTile)
        reinterpret_cast<uint4*>(s_w)[i] = __ldg(reinterpret_cast<const uint4*>(blob) + i);
    for (uint32_t i = tid; i < 2048 / 16; i += kTile) reinterpret_cast<uint4*>(s_slack)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 0) tmem_alloc(s_slot, 256);
    if (tid == 0) {
        mbar_init(s_bar, 1);
        mbar_fence_init();
    }
    const uint32_t row = blockIdx.x * kTile + tid;
    float q[14];
    load_query(in, nullptr, row, n, q);
    encode_row<IN>(ly, grid, q, s_act0, tid);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_slot;
    const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;
    uint32_t phase = 0;
    bool ok = true;

    // ---- forward
    for (int j = 0; j < L && ok; ++j) {
        if (tid == 0) {
            tc_fence_after();
            issue_layer(tmem, smem_u32(act(j)), smem_u32(s_w + ly.boff[j]), ly.in[j], ly.out[j]);
            mma_commit(s_bar);
        }
        ok = __syncthreads_and(mbar_wait(s_bar, phase));  // block-uniform decision
        phase ^= 1;
        tc_fence_after();
        if (!ok) break;
        if (j < L - 1) {
#pragma unroll
            for (int c = 0; c < kWidth / 16; ++c) {
                float v[16];
                tmem_ld16(tmem + lane_base + c * 16, v);
                tmem_wait_ld();
                store_row16_relu(act(j + 1), tid, c * 16, kWidth, v);
            }
        } else {
            // output, loss and its gradient (rows beyond n contribute nothing)
            float v[16];
            tmem_ld16(tmem + lane_base, v);
            tmem_wait_ld();
            float g[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) g[i] = 0.0f;
            float l = 0.0f;
            if (row < n) {
                float y[3], t[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    y[c] = ly.out_act == NRC_OUTPUT_EXP ? __expf(v[c]) : v[c];
                    t[c] = __ldg(target + static_cast<size_t>(row) * 3 + c);
                }
                float lum = 0.2126f * y[0] + 0.7152f * y[1] + 0.0722f * y[2];
                float denom = lum * lum + 0.01f;
                float inv = 1.0f / (3.0f * static_cast<float>(n));
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    float d = y[c] - t[c];
                    l += d * d / denom * inv;
                    float gy = 2.0f * d / denom * inv;
                    float gz = ly.out_act == NRC_OUTPUT_EXP ? gy * y[c] : gy;
                    g[c] = gz * ly.loss_scale;
                }
            }
            store_row16(s_dzo, tid, 0, kOutPad, g);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
            if ((tid & 31) == 0) atomicAdd(loss, l);
        }
        tc_fence_before();
        fence_async_smem();
        __syncthreads();
    }

    // ---- backward: for matrix j, dW_j = dPre_{j+1}^T act_j and dPre_j = (dPre_{j+1} W_j) * relu'(act_j)
    uint8_t* dz = s_dzo;
    uint8_t* dz_next = s_dza;
    const uint32_t tm_dx = tmem;        // columns [0, 64)
    const uint32_t tm_dw = tmem + 64;   // columns [64, 64 + in_j)
    for (int j = L - 1; j >= 0 && ok; --j) {
        const int K_out = ly.out[j], N_in = ly.in[j];
        if (tid == 0) {
            tc_fence_after();
            // weight gradient: M = 128 (output features, rows beyond out_j unused), N = in_j, K = 128 samples
            const uint32_t idw = idesc_f16(kTile, N_in, 1, 1);
            const uint64_t adw = smem_desc(smem_u32(dz), static_cast<uint32_t>(K_out * 16), 128);
            const uint64_t bdw = smem_desc(smem_u32(act(j)), static_cast<uint32_t>(N_in * 16), 128);
#pragma unroll
            for (int ks = 0; ks < kTile / 16; ++ks)  // 16 samples further: 2 K_out (2 N_in) in the address fields
                mma_f16(tm_dw, adw + 2 * K_out * ks, bdw + 2 * N_in * ks, idw, ks > 0 ? 1u : 0u);
            if (j > 0 || (IN == 64 && ly.enc == NRC_ENCODING_HASHGRID)) {
                // input gradient: M = 128 samples, N = in_j, K = out_j; W_j read MN-major
                const uint32_t idx = idesc_f16(kTile, N_in, 0, 1);
                const uint64_t adx = smem_desc(smem_u32(dz), 128, static_cast<uint32_t>(K_out * 16));
                const uint64_t bdx = smem_desc(smem_u32(s_w + ly.boff[j]), static_cast<uint32_t>(N_in * 16), 128);
                for (int ks = 0; ks < K_out / 16; ++ks)
                    mma_f16(tm_dx, adx + 16 * ks, bdx + 2 * N_in * ks, idx, ks > 0 ? 1u : 0u);
            }
            mma_commit(s_bar);
        }
        ok = __syncthreads_and(mbar_wait(s_bar, phase));  // block-uniform decision
        phase ^= 1;
        tc_fence_after();
        if (!ok) break;
        // Weight-gradient rows: TMEM lane = output feature. The TMEM load is warp-collective, so
        // every lane of a warp that holds gradient rows takes part; only real rows are reduced.
        const int out_real = j == L - 1 ? 3 : K_out;
        if (warp * 32 < out_real) {
            float* gdst = grad + ly.poff[j] + tid * N_in;
            for (int c = 0; c < N_in / 16; ++c) {
                float v[16];
                tmem_ld16(tm_dw + lane_base + c * 16, v);
                tmem_wait_ld();
                if (tid < out_real) {
#pragma unroll
                    for (int i = 0; i < 16; i += 4)
                        atomicAdd(reinterpret_cast<float4*>(gdst + c * 16 + i),
                                  make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]));
                }
            }
        }
        if (j > 0) {
#pragma unroll
            for (int c = 0; c < kWidth / 16; ++c) {
                float v[16], a[16];
                tmem_ld16(tm_dx + lane_base + c * 16, v);
                tmem_wait_ld();
                load_row16(act(j), tid, c * 16, kWidth, a);
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = a[i] > 0.0f ? v[i] : 0.0f;
                store_row16(dz_next, tid, c * 16, kWidth, v);
            }
            dz = dz_next;
            dz_next = dz_next == s_dza ? s_dzb : s_dza;
        } else if (IN == 64 && ly.enc == NRC_ENCODING_HASHGRID) {
            // gradient of the encoded input's hash features (columns 0..31) into the tables
            float a[16], b[16], d[32];
            tmem_ld16(tm_dx + lane_base, a);
            tmem_ld16(tm_dx + lane_base + 16, b);
            tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                d[i] = a[i];
                d[16 + i] = b[i];
            }
            if (row < n) grid_backward(ly, q, d, grad + ly.nparams);
        }
        tc_fence_before();
        fence_async_smem();
        __syncthreads();
    }
    if (!ok && tid == 0) atomicOr(err, kErrTimeout);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 256);
}

// ------------------------------------------------------------------------------ elementwise kernels
struct ParamIndex {
    int j, o, i;
};
__device__ __forceinline__ ParamIndex param_index(const NetLayout& ly, int p) {
    int j = 0;
    while (j + 1 < ly.L && p >= ly.poff[j + 1]) ++j;
    int r = p - ly.poff[j];
    return {j, r / ly.in[j], r % ly.in[j]};
}

// FP16 weight image in the shared-memory layout (matrix j as [out][in] core matrices).
__global__ void pack_kernel(const NetLayout ly, const float* __restrict__ w, uint8_t* __restrict__ blob) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= ly.nparams) return;
    ParamIndex x = param_index(ly, p);
    *reinterpret_cast<__half*>(blob + ly.boff[x.j] + cm_offset(x.o, x.i, ly.in[x.j])) = __float2half_rn(w[p]);
}

// FP16 image of the hash-grid tables (entry-major, two features per 32-bit word).
__global__ void pack_grid_kernel(const NetLayout ly, const float* __restrict__ w, __half* __restrict__ grid) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= ly.grid_params) return;
    grid[p] = __float2half_rn(w[ly.nparams + p]);
}

// Adam with L2 regularisation on unscaled gradients, optional EMA of the weights (inference
// weights = bias-corrected EMA), and repacking of both FP16 images. Parameters ly.nparams and
// beyond are hash-grid table entries (FP16 images grid_train / grid_infer); as published for the
// multiresolution hash encoding (Mueller et al. 2022, section 4), they take no L2 term and an
// entry whose gradient is exactly 0 skips its Adam step (its moments and value stay as they are).
__global__ void adam_kernel(const NetLayout ly, float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ grad, float* __restrict__ ema, uint8_t* __restrict__ blob_train,
                            uint8_t* __restrict__ blob_infer, __half* __restrict__ grid_train,
                            __half* __restrict__ grid_infer, float lr, float beta1, float beta2, float eps, float l2,
                            float inv_scale, float c1, float c2, float ema_decay, float ema_corr) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= ly.nparams + ly.grid_params) return;
    if (p >= ly.nparams) {
        float wi = w[p];
        const float gr = grad[p];
        if (gr != 0.0f) {
            float g = gr * inv_scale;
            float mi = beta1 * m[p] + (1.0f - beta1) * g;
            float vi = beta2 * v[p] + (1.0f - beta2) * g * g;
            m[p] = mi;
            v[p] = vi;
            wi -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
            w[p] = wi;
            grid_train[p - ly.nparams] = __float2half_rn(wi);
        }
        float wi_inf = wi;
        if (ema_decay > 0.0f) {
            float e = ema_decay * ema[p] + (1.0f - ema_decay) * wi;
            ema[p] = e;
            wi_inf = e / ema_corr;
        }
        grid_infer[p - ly.nparams] = __float2half_rn(wi_inf);
        return;
    }
    ParamIndex x = param_index(ly, p);
    bool real = x.i < (x.j == 0 ? ly.in_real : ly.in[x.j]) && x.o < (x.j == ly.L - 1 ? 3 : ly.out[x.j]);
    float wi = w[p];
    if (real) {
        float g = grad[p] * inv_scale + l2 * wi;
        float mi = beta1 * m[p] + (1.0f - beta1) * g;
        float vi = beta2 * v[p] + (1.0f - beta2) * g * g;
        m[p] = mi;
        v[p] = vi;
        wi -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[p] = wi;
    }
    uint32_t off = cm_offset(x.o, x.i, ly.in[x.j]);
    *reinterpret_cast<__half*>(blob_train + ly.boff[x.j] + off) = __float2half_rn(wi);
    float wi_inf = wi;
    if (ema_decay > 0.0f) {
        float e = ema_decay * ema[p] + (1.0f - ema_decay) * wi;
        ema[p] = e;
        wi_inf = e / ema_corr;
    }
    *reinterpret_cast<__half*>(blob_infer + ly.boff[x.j] + off) = __float2half_rn(wi_inf);
}

template <int IN>
__global__ void encode_kernel(const NetLayout ly, const uint32_t* __restrict__ grid, const float* __restrict__ in,
                              uint32_t n, float* __restrict__ out) {
    // Encodes one 128-row tile per CTA into shared memory, then writes FP32 rows.
    __shared__ __align__(128) uint8_t tile[kTile * IN * 2];
    uint32_t row = blockIdx.x * kTile + threadIdx.x;
    float q[14];
    load_query(in, nullptr, row, n, q);
    encode_row<IN>(ly, grid, q, tile, threadIdx.x);
    if (row < n)
        for (int c = 0; c < IN; c += 16) {
            float v[16];
            load_row16(tile, threadIdx.x, c, IN, v);
            for (int i = 0; i < 16; ++i) out[static_cast<size_t>(row) * IN + c + i] = v[i];
        }
}

// Issue rate of back-to-back MMAs from one thread (see nrc_selftest_mma_rate): M = 128, N = `n`,
// K = 16, both operands in shared memory (zeros), alternating between two accumulators.
__global__ void mma_rate_kernel(int n, uint32_t count, long long* __restrict__ out, unsigned int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sa = smem;             // 128 x 64 FP16, core-matrix layout
    uint8_t* sb = smem + 16384;     // 256 x 64 FP16
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 49152);
    uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < 49152 / 16; i += blockDim.x) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 0) tmem_alloc(slot, 512);
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    if (tid == 0) {
        const uint32_t idesc = idesc_f16(kTile, n, 0, 0);
        const uint64_t ad = smem_desc(smem_u32(sa), 128, 64 * 16);
        const uint64_t bd = smem_desc(smem_u32(sb), 128, 64 * 16);
        const long long t0 = clock64();
        for (uint32_t i = 0; i < count; i += 4) {
            const uint32_t d = tmem + ((i >> 2) & 1u) * 256u;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) mma_f16(d, ad + 16 * ks, bd + 16 * ks, idesc, (i > 0 || ks > 0) ? 1u : 0u);
        }
        mma_commit(bar);
        if (!mbar_wait(bar, 0)) atomicOr(err, kErrTimeout);
        out[0] = clock64() - t0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// Tensor-core self test (see nrc_selftest_mma).
__global__ void selftest_kernel(const float* __restrict__ A, const float* __restrict__ B, int a_mn, int b_mn,
                                float* __restrict__ D, unsigned int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr int M = 128, N = 64, K = 64;
    uint8_t* sa = smem;              // 16 KB
    uint8_t* sb = smem + 16384;      // 8 KB
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 65536);
    uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int e = tid; e < M * K; e += blockDim.x) {
        int m = e / K, k = e % K;
        uint32_t off = a_mn ? cm_offset(k, m, M) : cm_offset(m, k, K);
        *reinterpret_cast<__half*>(sa + off) = __float2half_rn(A[e]);
    }
    for (int e = tid; e < N * K; e += blockDim.x) {
        int nn = e / K, k = e % K;
        uint32_t off = b_mn ? cm_offset(k, nn, N) : cm_offset(nn, k, K);
        *reinterpret_cast<__half*>(sb + off) = __float2half_rn(B[e]);
    }
    if (warp == 0) tmem_alloc(slot, 64);
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    if (tid == 0) {
        // mode 1: MN-major with leading offset along K and stride offset along M/N (the kernels'
        // convention); mode 2: the two offsets exchanged (diagnostic).
        const uint32_t id = idesc_f16(M, N, a_mn ? 1 : 0, b_mn ? 1 : 0);
        for (int ks = 0; ks < K / 16; ++ks) {
            uint64_t ad = a_mn == 1   ? smem_desc(smem_u32(sa) + ks * 2 * (M * 16), M * 16, 128)
                          : a_mn == 2 ? smem_desc(smem_u32(sa) + ks * 2 * (M * 16), 128, M * 16)
                                      : smem_desc(smem_u32(sa) + ks * 256, 128, K * 16);
            uint64_t bd = b_mn == 1   ? smem_desc(smem_u32(sb) + ks * 2 * (N * 16), N * 16, 128)
                          : b_mn == 2 ? smem_desc(smem_u32(sb) + ks * 2 * (N * 16), 128, N * 16)
                                      : smem_desc(smem_u32(sb) + ks * 256, 128, K * 16);
            mma_f16(tmem, ad, bd, id, ks > 0 ? 1u : 0u);
        }
        mma_commit(bar);
    }
    bool ok = __syncthreads_and(mbar_wait(bar, 0));
    tc_fence_after();
    if (ok) {
        for (int c = 0; c < N / 16; ++c) {
            float v[16];
            tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + c * 16, v);
            tmem_wait_ld();
            for (int i = 0; i < 16; ++i) D[tid * N + c * 16 + i] = v[i];
        }
    } else if (tid == 0) {
        atomicOr(err, kErrTimeout);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 64);
}

// ------------------------------------------------------------------------------ host side
// Hidden activations in tensor memory (the TA form of the inference kernel).
constexpr bool kInferTmemActivations = true;
constexpr uint32_t kMaxSmemOptIn = 232448;  // 227 KB per CTA
uint32_t infer_smem(const NetLayout& l, int groups) {
    const uint32_t s = align_up(l.blob_bytes, 1024) + groups * infer_tile_bytes(l.in_dim) + groups * 8 + 16;
    // The TA form allocates 128 TMEM columns per group, all 512 of an SM at four groups: the
    // shared-memory request keeps a second CTA off the SM so that its allocation never waits.
    return kInferTmemActivations ? std::max<uint32_t>(s, kMaxSmemOptIn / 2 + 1024) : s;
}
// Largest tile-group count (4, 2 or 1) whose shared memory fits one CTA.
int infer_groups(const NetLayout& l) {
    for (int g = 4; g > 1; g /= 2)
        if (infer_smem(l, g) <= kMaxSmemOptIn) return g;
    return 1;
}
const void* infer_kernel_ptr(int enc, int groups) {
    const bool vol = enc == NRC_ENCODING_VOLUME;
    switch (groups) {
    case 4: return vol ? reinterpret_cast<const void*>(mlp_infer_kernel<144, 4, kInferTmemActivations>)
                       : reinterpret_cast<const void*>(mlp_infer_kernel<64, 4, kInferTmemActivations>);
    case 2: return vol ? reinterpret_cast<const void*>(mlp_infer_kernel<144, 2, kInferTmemActivations>)
                       : reinterpret_cast<const void*>(mlp_infer_kernel<64, 2, kInferTmemActivations>);
    default: return vol ? reinterpret_cast<const void*>(mlp_infer_kernel<144, 1, kInferTmemActivations>)
                        : reinterpret_cast<const void*>(mlp_infer_kernel<64, 1, kInferTmemActivations>);
    }
}
uint32_t train_smem(const NetLayout& l) {
    return align_up(l.blob_bytes, 1024) + kTile * l.in_dim * 2 + (l.L - 1) * kTile * kWidth * 2 +
           2 * kTile * kWidth * 2 + kTile * kOutPad * 2 + 2048 + 16;
}

}  // namespace
}  // namespace nrc

using namespace nrc;

struct NrcHandle {
    NrcConfig cfg;
    NetLayout ly;
    int num_sms = 0;
    int infer_groups = 1;  // 128-row tiles in flight per inference CTA
    float *w = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *ema = nullptr, *loss = nullptr;
    uint8_t *blob_train = nullptr, *blob_infer = nullptr;
    __half *grid_train = nullptr, *grid_infer = nullptr;  // FP16 hash-grid tables (hash grid only)
    unsigned int* err = nullptr;
    uint64_t steps = 0;
    int total_params() const { return ly.nparams + ly.grid_params; }
    const uint32_t* grid_words(bool train) const {
        return reinterpret_cast<const uint32_t*>(train ? grid_train : grid_infer);
    }
};

namespace {
template <typename T>
int alloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
    if (e != cudaSuccess) return fail(NRC_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return NRC_OK;
}

int set_kernel_smem(const void* k, uint32_t bytes) {
    NRC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
    return NRC_OK;
}

int repack(NrcHandle* h, cudaStream_t s) {
    int n = h->ly.nparams;
    pack_kernel<<<(n + 255) / 256, 256, 0, s>>>(h->ly, h->w, h->blob_train);
    pack_kernel<<<(n + 255) / 256, 256, 0, s>>>(h->ly, h->cfg.ema_decay > 0 ? h->ema : h->w, h->blob_infer);
    if (h->ly.grid_params > 0) {
        const int g = h->ly.grid_params;
        pack_grid_kernel<<<(g + 255) / 256, 256, 0, s>>>(h->ly, h->w, h->grid_train);
        pack_grid_kernel<<<(g + 255) / 256, 256, 0, s>>>(h->ly, h->cfg.ema_decay > 0 ? h->ema : h->w, h->grid_infer);
    }
    NRC_CUDA(cudaGetLastError());
    return NRC_OK;
}
}  // namespace

extern "C" {

const char* nrc_last_error(void) { return g_err.c_str(); }

void nrc_default_config(int32_t encoding, NrcConfig* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->encoding = encoding;
    c->beta1 = 0.9f;
    c->beta2 = 0.99f;
    c->learning_rate = 1e-2f;
    c->loss_scale = 128.0f;
    c->seed = 1;
    if (encoding == NRC_ENCODING_REFERENCE || encoding == NRC_ENCODING_HASHGRID) {
        // network_interface.cu:50-122: 2 hidden layers (renderer_scene.cpp:50), EMA 0.99, l2 1e-6,
        // output activation None; Adam epsilon 1e-8 with TriangleWave, 1e-15 with the hash grid.
        c->num_hidden_layers = 2;
        c->epsilon = encoding == NRC_ENCODING_HASHGRID ? 1e-15f : 1e-8f;
        c->l2_reg = 1e-6f;
        c->ema_decay = 0.99f;
        c->output_activation = NRC_OUTPUT_NONE;
    } else {
        // The volume cache: 5 hidden layers, exp output, Adam lr 1e-2, betas 0.9 / 0.99.
        c->num_hidden_layers = 5;
        c->epsilon = 1e-8f;
        c->l2_reg = 0.0f;
        c->ema_decay = 0.0f;
        c->output_activation = NRC_OUTPUT_EXP;
    }
}

int nrc_create(const NrcConfig* cfg, NrcHandle** out) {
    if (!cfg || !out) return fail(NRC_ERR_INVALID_ARGUMENT, "nrc_create: null argument");
    if (cfg->encoding != NRC_ENCODING_REFERENCE && cfg->encoding != NRC_ENCODING_VOLUME &&
        cfg->encoding != NRC_ENCODING_HASHGRID)
        return fail(NRC_ERR_INVALID_ARGUMENT, "nrc_create: unknown encoding");
    int max_hidden = cfg->encoding == NRC_ENCODING_VOLUME ? 5 : 7;  // training tile must fit in shared memory
    if (cfg->num_hidden_layers < 1 || cfg->num_hidden_layers > max_hidden)
        return fail(NRC_ERR_INVALID_ARGUMENT,
                    "nrc_create: num_hidden_layers out of range (1..5 volume, 1..7 reference and hash grid)");
    if (!(cfg->learning_rate > 0) || !(cfg->loss_scale > 0) || cfg->ema_decay < 0 || cfg->ema_decay >= 1)
        return fail(NRC_ERR_INVALID_ARGUMENT, "nrc_create: bad optimiser settings");
    auto* h = new NrcHandle();
    h->cfg = *cfg;
    h->ly = make_layout(cfg->encoding, cfg->num_hidden_layers, cfg->output_activation, cfg->loss_scale);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev);
    const int np = h->total_params();
    const int ng = std::max(h->ly.grid_params, 2);
    int rc;
    if ((rc = alloc(&h->w, np)) || (rc = alloc(&h->m, np)) || (rc = alloc(&h->v, np)) || (rc = alloc(&h->grad, np)) ||
        (rc = alloc(&h->ema, np)) || (rc = alloc(&h->loss, 1)) || (rc = alloc(&h->blob_train, h->ly.blob_bytes)) ||
        (rc = alloc(&h->blob_infer, h->ly.blob_bytes)) || (rc = alloc(&h->grid_train, ng)) ||
        (rc = alloc(&h->grid_infer, ng)) || (rc = alloc(&h->err, 1))) {
        nrc_destroy(h);
        return rc;
    }
    // Uniform initialisation with bound sqrt(6 / (fan_in + fan_out)); padded rows/columns are 0.
    std::vector<float> w(np, 0.0f);
    std::mt19937 gen(cfg->seed);
    for (int j = 0; j < h->ly.L; ++j) {
        int in_real = j == 0 ? h->ly.in_real : h->ly.in[j];
        int out_real = j == h->ly.L - 1 ? 3 : h->ly.out[j];
        float bound = std::sqrt(6.0f / static_cast<float>(in_real + out_real));
        std::uniform_real_distribution<float> u(-bound, bound);
        for (int o = 0; o < out_real; ++o)
            for (int i = 0; i < in_real; ++i) w[h->ly.poff[j] + o * h->ly.in[j] + i] = u(gen);
    }
    // Hash-grid entries start uniform in [-1e-4, 1e-4] (the published initialisation).
    std::uniform_real_distribution<float> ug(-1e-4f, 1e-4f);
    for (int p = h->ly.nparams; p < np; ++p) w[p] = ug(gen);
    if (cudaMemcpy(h->w, w.data(), np * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(h->m, 0, np * sizeof(float)) != cudaSuccess || cudaMemset(h->v, 0, np * sizeof(float)) != cudaSuccess ||
        cudaMemset(h->grad, 0, np * sizeof(float)) != cudaSuccess ||
        cudaMemset(h->ema, 0, np * sizeof(float)) != cudaSuccess || cudaMemset(h->err, 0, sizeof(unsigned int)) != cudaSuccess) {
        nrc_destroy(h);
        return fail(NRC_ERR_CUDA, "nrc_create: initial upload failed");
    }
    if (cfg->ema_decay > 0)
        cudaMemcpy(h->ema, w.data(), np * sizeof(float), cudaMemcpyHostToDevice);
    if ((rc = repack(h, 0))) {
        nrc_destroy(h);
        return rc;
    }
    const bool vol = cfg->encoding == NRC_ENCODING_VOLUME;
    h->infer_groups = infer_groups(h->ly);
    if ((rc = set_kernel_smem(infer_kernel_ptr(cfg->encoding, h->infer_groups), infer_smem(h->ly, h->infer_groups))) ||
        (rc = set_kernel_smem(vol ? reinterpret_cast<const void*>(mlp_train_kernel<144>)
                                  : reinterpret_cast<const void*>(mlp_train_kernel<64>),
                              train_smem(h->ly)))) {
        nrc_destroy(h);
        return rc;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
        nrc_destroy(h);
        return fail(NRC_ERR_CUDA, "nrc_create: initialisation failed");
    }
    *out = h;
    return NRC_OK;
}

int nrc_destroy(NrcHandle* h) {
    if (!h) return NRC_OK;
    cudaFree(h->w);
    cudaFree(h->m);
    cudaFree(h->v);
    cudaFree(h->grad);
    cudaFree(h->ema);
    cudaFree(h->loss);
    cudaFree(h->blob_train);
    cudaFree(h->blob_infer);
    cudaFree(h->grid_train);
    cudaFree(h->grid_infer);
    cudaFree(h->err);
    delete h;
    return NRC_OK;
}

static int infer_impl(NrcHandle* h, void* stream, const float* in, const uint32_t* idx, const uint32_t* dev_n,
                      uint32_t n, float* out) {
    if (!h || !in || !out) return fail(NRC_ERR_INVALID_ARGUMENT, "nrc_infer: null argument");
    if (n == 0) return NRC_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int G = h->infer_groups;
    const uint32_t tiles = (n + kTile - 1) / kTile;
    const uint32_t grid = std::min<uint32_t>((tiles + G - 1) / G, static_cast<uint32_t>(h->num_sms));
    const uint32_t smem = infer_smem(h->ly, G);
    const bool vol = h->cfg.encoding == NRC_ENCODING_VOLUME;
    const dim3 block(kTile * G);
    const uint32_t* gw = h->grid_words(false);
    if (G == 4) {
        if (vol)
            mlp_infer_kernel<144, 4, kInferTmemActivations><<<grid, block, smem, s>>>(h->ly, h->blob_infer, gw, in, idx, dev_n, n, out, h->err);
        else
            mlp_infer_kernel<64, 4, kInferTmemActivations><<<grid, block, smem, s>>>(h->ly, h->blob_infer, gw, in, idx, dev_n, n, out, h->err);
    } else if (G == 2) {
        if (vol)
            mlp_infer_kernel<144, 2, kInferTmemActivations><<<grid, block, smem, s>>>(h->ly, h->blob_infer, gw, in, idx, dev_n, n, out, h->err);
        else
            mlp_infer_kernel<64, 2, kInferTmemActivations><<<grid, block, smem, s>>>(h->ly, h->blob_infer, gw, in, idx, dev_n, n, out, h->err);
    } else {
        if (vol)
            mlp_infer_kernel<144, 1, kInferTmemActivations><<<grid, block, smem, s>>>(h->ly, h->blob_infer, gw, in, idx, dev_n, n, out, h->err);
        else
            mlp_infer_kernel<64, 1, kInferTmemActivations><<<grid, block, smem, s>>>(h->ly, h->blob_infer, gw, in, idx, dev_n, n, out, h->err);
    }
    NRC_CUDA(cudaGetLastError());
    return NRC_OK;
}

int nrc_infer(NrcHandle* h, void* stream, const float* in, uint32_t n, float* out) {
    return infer_impl(h, stream, in, nullptr, nullptr, n, out);
}

int nrc_infer_device_count(NrcHandle* h, void* stream, const float* in, const uint32_t* dev_n, uint32_t n_max,
                           float* out) {
    if (!dev_n) return fail(NRC_ERR_INVALID_ARGUMENT, "nrc_infer_device_count: null count");
    return infer_impl(h, stream, in, nullptr, dev_n, n_max, out);
}

int nrc_infer_indexed(NrcHandle* h, void* stream, const float* in, const uint32_t* idx, const uint32_t* dev_n,
                      uint32_t n_max, float* out) {
    if (!idx || !dev_n) return fail(NRC_ERR_INVALID_ARGUMENT, "nrc_infer_indexed: null index list or count");
    return infer_impl(h, stream, in, idx, dev_n, n_max, out);
}

int nrc_train(NrcHandle* h, void* stream, const float* in, const float* target, uint32_t n, float* loss_out) {
    if (!h || !in || !target) return fail(NRC_ERR_INVALID_ARGUMENT, "nrc_train: null argument");
    if (n == 0) return NRC_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const NetLayout& ly = h->ly;
    const int np = h->total_params();
    NRC_CUDA(cudaMemsetAsync(h->grad, 0, np * sizeof(float), s));
    NRC_CUDA(cudaMemsetAsync(h->loss, 0, sizeof(float), s));
    uint32_t tiles = (n + kTile - 1) / kTile;
    uint32_t smem = train_smem(ly);
    const uint32_t* gw = h->grid_words(true);
    if (h->cfg.encoding == NRC_ENCODING_VOLUME)
        mlp_train_kernel<144><<<tiles, kTile, smem, s>>>(ly, h->blob_train, gw, in, target, n, h->grad, h->loss, h->err);
    else
        mlp_train_kernel<64><<<tiles, kTile, smem, s>>>(ly, h->blob_train, gw, in, target, n, h->grad, h->loss, h->err);
    ++h->steps;
    const NrcConfig& c = h->cfg;
    float c1 = 1.0f - std::pow(c.beta1, static_cast<float>(h->steps));
    float c2 = 1.0f - std::pow(c.beta2, static_cast<float>(h->steps));
    // The EMA starts from the initial weights (not from zero), so it needs no bias correction.
    const float ema_corr = 1.0f;
    adam_kernel<<<(np + 255) / 256, 256, 0, s>>>(ly, h->w, h->m, h->v, h->grad, h->ema, h->blob_train, h->blob_infer,
                                                 h->grid_train, h->grid_infer, c.learning_rate, c.beta1, c.beta2,
                                                 c.epsilon, c.l2_reg, 1.0f / c.loss_scale, c1, c2, c.ema_decay,
                                                 ema_corr);
    NRC_CUDA(cudaGetLastError());
    if (loss_out) {
        NRC_CUDA(cudaMemcpyAsync(loss_out, h->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
        NRC_CUDA(cudaStreamSynchronize(s));
    }
    return NRC_OK;
}

int nrc_get_layout(NrcHandle* h, int32_t* num_layers, int32_t* in_dims, int32_t* out_dims, int64_t* total) {
    if (!h) return fail(NRC_ERR_INVALID_ARGUMENT, "null handle");
    if (num_layers) *num_layers = h->ly.L;
    for (int j = 0; j < h->ly.L; ++j) {
        if (in_dims) in_dims[j] = h->ly.in[j];
        if (out_dims) out_dims[j] = h->ly.out[j];
    }
    if (total) *total = h->total_params();
    return NRC_OK;
}

int nrc_get_params(NrcHandle* h, float* host) {
    if (!h || !host) return fail(NRC_ERR_INVALID_ARGUMENT, "null argument");
    NRC_CUDA(cudaDeviceSynchronize());
    NRC_CUDA(cudaMemcpy(host, h->w, h->total_params() * sizeof(float), cudaMemcpyDeviceToHost));
    return NRC_OK;
}

int nrc_set_params(NrcHandle* h, const float* host) {
    if (!h || !host) return fail(NRC_ERR_INVALID_ARGUMENT, "null argument");
    NRC_CUDA(cudaDeviceSynchronize());
    NRC_CUDA(cudaMemcpy(h->w, host, h->total_params() * sizeof(float), cudaMemcpyHostToDevice));
    NRC_CUDA(cudaMemcpy(h->ema, host, h->total_params() * sizeof(float), cudaMemcpyHostToDevice));
    int rc = repack(h, 0);
    if (rc) return rc;
    NRC_CUDA(cudaDeviceSynchronize());
    return NRC_OK;
}

int nrc_get_gradients(NrcHandle* h, float* host) {
    if (!h || !host) return fail(NRC_ERR_INVALID_ARGUMENT, "null argument");
    NRC_CUDA(cudaDeviceSynchronize());
    NRC_CUDA(cudaMemcpy(host, h->grad, h->total_params() * sizeof(float), cudaMemcpyDeviceToHost));
    const float inv = 1.0f / h->cfg.loss_scale;
    for (int i = 0; i < h->total_params(); ++i) host[i] *= inv;
    return NRC_OK;
}

int nrc_encode(NrcHandle* h, void* stream, const float* in, uint32_t n, float* out) {
    if (!h || !in || !out) return fail(NRC_ERR_INVALID_ARGUMENT, "null argument");
    if (n == 0) return NRC_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t tiles = (n + kTile - 1) / kTile;
    if (h->cfg.encoding == NRC_ENCODING_VOLUME)
        encode_kernel<144><<<tiles, kTile, 0, s>>>(h->ly, h->grid_words(true), in, n, out);
    else
        encode_kernel<64><<<tiles, kTile, 0, s>>>(h->ly, h->grid_words(true), in, n, out);
    NRC_CUDA(cudaGetLastError());
    return NRC_OK;
}

uint64_t nrc_step_count(NrcHandle* h) { return h ? h->steps : 0; }

uint32_t nrc_device_errors(NrcHandle* h) {
    if (!h) return 0;
    unsigned int e = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) return 0xffffffffu;
    if (cudaMemcpy(&e, h->err, sizeof(e), cudaMemcpyDeviceToHost) != cudaSuccess) return 0xffffffffu;
    cudaMemset(h->err, 0, sizeof(unsigned int));
    return e;
}

int nrc_selftest_mma_rate(int32_t n, uint32_t count, double* cycles_per_mma) {
    if (!cycles_per_mma || n < 16 || n > 256 || n % 16 || count == 0 || count > 65536)
        return fail(NRC_ERR_INVALID_ARGUMENT, "nrc_selftest_mma_rate: n must be a multiple of 16 in [16, 256], "
                                              "count in [1, 65536]");
    count = (count + 3) / 4 * 4;
    long long* dout = nullptr;
    unsigned int* derr = nullptr;
    int rc;
    if ((rc = alloc(&dout, 1)) || (rc = alloc(&derr, 1))) {
        cudaFree(dout);
        return rc;
    }
    cudaMemset(derr, 0, sizeof(unsigned int));
    const uint32_t smem = 49152 + 64;
    cudaFuncSetAttribute(mma_rate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    mma_rate_kernel<<<1, 128, smem>>>(n, count, dout, derr);
    cudaError_t e = cudaDeviceSynchronize();
    long long cyc = 0;
    unsigned int herr = 0;
    if (e == cudaSuccess) {
        cudaMemcpy(&cyc, dout, sizeof(cyc), cudaMemcpyDeviceToHost);
        cudaMemcpy(&herr, derr, sizeof(herr), cudaMemcpyDeviceToHost);
    }
    cudaFree(dout);
    cudaFree(derr);
    if (e != cudaSuccess) return fail(NRC_ERR_CUDA, std::string("selftest: ") + cudaGetErrorString(e));
    if (herr) return fail(NRC_ERR_DEVICE, "selftest: tensor-core completion wait timed out");
    *cycles_per_mma = static_cast<double>(cyc) / count;
    return NRC_OK;
}

int nrc_selftest_mma(const float* a, const float* b, int32_t a_mn, int32_t b_mn, float* d) {
    if (!a || !b || !d) return fail(NRC_ERR_INVALID_ARGUMENT, "null argument");
    float *da = nullptr, *db = nullptr, *dd = nullptr;
    unsigned int* derr = nullptr;
    int rc;
    if ((rc = alloc(&da, 128 * 64)) || (rc = alloc(&db, 64 * 64)) || (rc = alloc(&dd, 128 * 64)) || (rc = alloc(&derr, 1)))
        return rc;
    cudaMemcpy(da, a, 128 * 64 * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(db, b, 64 * 64 * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(derr, 0, sizeof(unsigned int));
    const uint32_t smem = 65536 + 64;
    cudaFuncSetAttribute(selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    selftest_kernel<<<1, 128, smem>>>(da, db, std::min(std::max(a_mn, 0), 2), std::min(std::max(b_mn, 0), 2), dd, derr);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned int herr = 0;
    if (e == cudaSuccess) {
        cudaMemcpy(d, dd, 128 * 64 * sizeof(float), cudaMemcpyDeviceToHost);
        cudaMemcpy(&herr, derr, sizeof(herr), cudaMemcpyDeviceToHost);
    }
    cudaFree(da);
    cudaFree(db);
    cudaFree(dd);
    cudaFree(derr);
    if (e != cudaSuccess) return fail(NRC_ERR_CUDA, std::string("selftest: ") + cudaGetErrorString(e));
    if (herr) return fail(NRC_ERR_DEVICE, "selftest: tensor-core completion wait timed out");
    return NRC_OK;
}

}  // extern "C"
