/*
 * ORACLE (test infrastructure only) — CPU restatement of the neural radiance cache network
 * used to check the GPU MLP kernels: input encodings, forward pass, relative-L2-luminance loss,
 * backward pass and the Adam update, in double precision with FP16 rounding at exactly the
 * points where the GPU stores FP16 values (encoded input, weights, hidden activations, scaled
 * output / hidden gradients).
 *
 * Parity status: the reference's network lives in tiny-cuda-nn (renderer/network_interface.cu:
 * 50-192, an un-vendored submodule whose pinned commit is not recorded in this checkout), so
 * the network is parity unpinned against the reference; these routines pin the GPU kernels to
 * the published algorithms they implement (one-blob / frequency / triangle-wave encodings, the
 * multiresolution hash encoding of Mueller et al. 2022 with the reference's HashGrid settings
 * (network_interface.cu:99-109: 16 levels x 2 features, 2^15 entries, base resolution 16,
 * per-level scale 2), ReLU MLP, Adam with L2 regularisation, relative L2 loss with a
 * stop-gradient denominator).
 *
 * Encodings: 0 = TriangleWave(12) + OneBlob(4) + identity (64 inputs), 1 = the volume encoding
 * (144 inputs), 2 = HashGrid + OneBlob(4) + identity (64 inputs). With the hash grid the
 * parameter vector is the MLP matrices followed by the tables (level by level, entry by entry,
 * two features per entry).
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int kWidth = 64;
constexpr int kOutPad = 16;

inline float h16(float x) { return static_cast<float>(static_cast<_Float16>(x)); }

int in_dim(int encoding) { return encoding == 1 ? 144 : 64; }

// ---- multiresolution hash grid
constexpr int kLevels = 16;
struct GridLevels {
    float scale[kLevels];
    uint32_t res[kLevels], size[kLevels], off[kLevels];
    bool hashed[kLevels];
    int64_t params;  // 2 x entries
};
GridLevels grid_levels() {
    GridLevels g{};
    uint32_t off = 0;
    for (int l = 0; l < kLevels; ++l) {
        // scale 16 * 2^l - 1, resolution ceil(scale) + 1, min(res^3 rounded up to 8, 2^15) entries
        g.scale[l] = std::exp2(static_cast<float>(l)) * 16.0f - 1.0f;
        g.res[l] = static_cast<uint32_t>(std::ceil(g.scale[l])) + 1u;
        const uint64_t cells = static_cast<uint64_t>(g.res[l]) * g.res[l] * g.res[l];
        const uint64_t padded = (cells + 7) / 8 * 8;
        g.size[l] = static_cast<uint32_t>(std::min<uint64_t>(padded, 1u << 15));
        g.hashed[l] = cells > g.size[l];
        g.off[l] = off;
        off += g.size[l];
    }
    g.params = 2 * static_cast<int64_t>(off);
    return g;
}
const GridLevels kGrid = grid_levels();

// Corner c of level l around position p (in [0,1]^3 after clamping): table entry and weight.
void grid_corners(int l, const float* q, uint32_t e[8], float w[8]) {
    float fr[3];
    uint32_t g[3];
    for (int d = 0; d < 3; ++d) {
        const float x = std::min(std::max(q[d], 0.0f), 1.0f);
        const float pos = std::fma(kGrid.scale[l], x, 0.5f);
        const float fl = std::floor(pos);
        fr[d] = pos - fl;
        g[d] = static_cast<uint32_t>(static_cast<int>(fl));
    }
    for (int c = 0; c < 8; ++c) {
        const uint32_t x = g[0] + (c & 1), y = g[1] + ((c >> 1) & 1), z = g[2] + ((c >> 2) & 1);
        const float wx = (c & 1) ? fr[0] : 1.0f - fr[0];
        const float wy = (c & 2) ? fr[1] : 1.0f - fr[1];
        const float wz = (c & 4) ? fr[2] : 1.0f - fr[2];
        w[c] = (wx * wy) * wz;
        const uint32_t res = kGrid.res[l];
        const uint32_t i = kGrid.hashed[l] ? (x ^ (y * 2654435761u) ^ (z * 805459861u)) : (x + (y + z * res) * res);
        e[c] = kGrid.off[l] + i % kGrid.size[l];
    }
}

// Encoded network input of one query (padded with zeros), as floats before FP16 rounding.
// `grid` = the hash-grid tables (encoding 2 only), read through FP16 as the GPU does.
void encode(int encoding, const float* q, float* out, const float* grid = nullptr) {
    int d = in_dim(encoding);
    for (int i = 0; i < d; ++i) out[i] = 0.0f;
    int k = 0;
    if (encoding == 2) {
        for (int l = 0; l < kLevels; ++l) {
            uint32_t e[8];
            float w[8];
            grid_corners(l, q, e, w);
            for (int f = 0; f < 2; ++f) {
                double acc = 0.0;
                for (int c = 0; c < 8; ++c) acc += static_cast<double>(w[c]) * h16(grid[2 * e[c] + f]);
                out[k++] = static_cast<float>(acc);
            }
        }
        const float scale[5] = {1.0f / 3.14159265f, 1.0f / 6.28318531f, 1.0f / 3.14159265f, 1.0f / 6.28318531f, 1.0f};
        for (int a = 0; a < 5; ++a) {
            float x = q[3 + a] * scale[a];
            for (int b = 0; b < 4; ++b) {
                float z = (x - (b + 0.5f) / 4.0f) * 4.0f;
                out[k++] = std::exp(-0.5f * z * z);
            }
        }
        for (int a = 0; a < 6; ++a) out[k++] = q[8 + a];
        return;
    }
    if (encoding == 0) {
        for (int a = 0; a < 3; ++a)
            for (int f = 0; f < 12; ++f) {
                float v = q[a] * static_cast<float>(1 << f);
                float fr = v - std::floor(v);
                out[k++] = 2.0f * std::fabs(fr - 0.5f);
            }
        const float scale[5] = {1.0f / 3.14159265f, 1.0f / 6.28318531f, 1.0f / 3.14159265f, 1.0f / 6.28318531f, 1.0f};
        for (int a = 0; a < 5; ++a) {
            float x = q[3 + a] * scale[a];
            for (int b = 0; b < 4; ++b) {
                float z = (x - (b + 0.5f) / 4.0f) * 4.0f;
                out[k++] = std::exp(-0.5f * z * z);
            }
        }
        for (int a = 0; a < 6; ++a) out[k++] = q[8 + a];
    } else {
        for (int a = 0; a < 3; ++a)
            for (int f = 0; f < 12; ++f) {
                // sin / cos of pi * (x * 2^f), with the product x * 2^f exact in float
                double arg = kPi * static_cast<double>(q[a] * static_cast<float>(1 << f));
                out[k++] = static_cast<float>(std::sin(arg));
                out[k++] = static_cast<float>(std::cos(arg));
            }
        const float scale[2] = {1.0f / 3.14159265f, 1.0f / 6.28318531f};
        for (int a = 0; a < 2; ++a) {
            float x = q[5 + a] * scale[a];
            for (int b = 0; b < 32; ++b) {
                float z = (x - (b + 0.5f) / 32.0f) * 32.0f;
                out[k++] = std::exp(-0.5f * z * z);
            }
        }
        out[k++] = q[7];
        out[k++] = q[8];
    }
}

struct Layout {
    int L;                 // number of weight matrices
    std::vector<int> in, out;
    std::vector<int64_t> off;
    int64_t total;         // MLP weights and (hash grid) the tables after them
    int64_t mlp;           // MLP weights
};
Layout layout(int encoding, int hidden) {
    Layout l;
    l.L = hidden + 1;
    for (int i = 0; i < l.L; ++i) {
        l.in.push_back(i == 0 ? in_dim(encoding) : kWidth);
        l.out.push_back(i == l.L - 1 ? kOutPad : kWidth);
    }
    int64_t o = 0;
    for (int i = 0; i < l.L; ++i) {
        l.off.push_back(o);
        o += static_cast<int64_t>(l.in[i]) * l.out[i];
    }
    l.mlp = o;
    l.total = o + (encoding == 2 ? kGrid.params : 0);
    return l;
}

inline double lum(const double* y) { return 0.2126 * y[0] + 0.7152 * y[1] + 0.0722 * y[2]; }

}  // namespace

extern "C" {

int orc_nrc_in_dim(int encoding) { return in_dim(encoding); }

int64_t orc_nrc_num_params(int encoding, int hidden) { return layout(encoding, hidden).total; }

// `grid` = the hash-grid tables (encoding 2), else ignored.
void orc_nrc_encode(int encoding, const float* in, int n, float* out, const float* grid) {
    int d = in_dim(encoding);
    for (int i = 0; i < n; ++i) encode(encoding, in + 14 * i, out + static_cast<int64_t>(d) * i, grid);
}

int64_t orc_nrc_grid_params(void) { return kGrid.params; }

// Forward pass; `acts` (optional) receives the FP16-rounded activations of every layer input.
void orc_nrc_forward(int encoding, int hidden, int out_act, const float* params, const float* in, int n, float* out) {
    Layout ly = layout(encoding, hidden);
    std::vector<float> x(256), y(256);
    for (int i = 0; i < n; ++i) {
        encode(encoding, in + 14 * i, x.data(), params + ly.mlp);
        for (int k = 0; k < ly.in[0]; ++k) x[k] = h16(x[k]);
        for (int l = 0; l < ly.L; ++l) {
            const float* W = params + ly.off[l];
            for (int o = 0; o < ly.out[l]; ++o) {
                double acc = 0.0;
                for (int k = 0; k < ly.in[l]; ++k) acc += static_cast<double>(h16(W[o * ly.in[l] + k])) * x[k];
                y[o] = static_cast<float>(acc);
            }
            if (l < ly.L - 1) {
                for (int o = 0; o < ly.out[l]; ++o) x[o] = h16(std::max(y[o], 0.0f));
            }
        }
        for (int c = 0; c < 3; ++c) out[3 * i + c] = out_act == 1 ? std::exp(y[c]) : y[c];
    }
}

// Loss and parameter gradients of one training batch (the GPU's nrc_train semantics).
double orc_nrc_loss_grad(int encoding, int hidden, int out_act, float loss_scale, const float* params,
                         const float* in, const float* target, int n, float* grads) {
    Layout ly = layout(encoding, hidden);
    std::vector<double> g(ly.total, 0.0);
    double loss = 0.0;
    std::vector<std::vector<float>> acts(ly.L + 1, std::vector<float>(256));
    std::vector<float> pre(256);
    std::vector<double> dz(256), dnext(256);
    for (int i = 0; i < n; ++i) {
        std::vector<float>& x0 = acts[0];
        encode(encoding, in + 14 * i, x0.data(), params + ly.mlp);
        for (int k = 0; k < ly.in[0]; ++k) x0[k] = h16(x0[k]);
        double yout[kOutPad];
        for (int l = 0; l < ly.L; ++l) {
            const float* W = params + ly.off[l];
            for (int o = 0; o < ly.out[l]; ++o) {
                double acc = 0.0;
                for (int k = 0; k < ly.in[l]; ++k) acc += static_cast<double>(h16(W[o * ly.in[l] + k])) * acts[l][k];
                if (l < ly.L - 1)
                    acts[l + 1][o] = h16(std::max(static_cast<float>(acc), 0.0f));
                else
                    yout[o] = static_cast<float>(acc);
            }
        }
        double y[3], t[3];
        for (int c = 0; c < 3; ++c) {
            y[c] = out_act == 1 ? std::exp(static_cast<float>(yout[c])) : yout[c];
            t[c] = target[3 * i + c];
        }
        double denom = lum(y) * lum(y) + 0.01;
        // Output gradient (scaled, FP16 like the GPU's output-gradient tile).
        for (int o = 0; o < kOutPad; ++o) dz[o] = 0.0;
        for (int c = 0; c < 3; ++c) {
            double d = y[c] - t[c];
            loss += d * d / denom / (3.0 * n);
            double gy = 2.0 * d / denom / (3.0 * n);
            double gz = out_act == 1 ? gy * y[c] : gy;
            dz[c] = h16(static_cast<float>(gz * loss_scale));
        }
        for (int l = ly.L - 1; l >= 0; --l) {
            const float* W = params + ly.off[l];
            // weight gradient
            for (int o = 0; o < ly.out[l]; ++o) {
                if (dz[o] == 0.0) continue;
                for (int k = 0; k < ly.in[l]; ++k) g[ly.off[l] + o * ly.in[l] + k] += dz[o] * acts[l][k];
            }
            if (l == 0 && encoding == 2) {
                // gradient of the 32 hash features, spread over each level's 8 corners
                const float* q = in + 14 * i;
                for (int lv = 0; lv < kLevels; ++lv) {
                    double dx[2];
                    for (int f = 0; f < 2; ++f) {
                        double acc = 0.0;
                        for (int o = 0; o < ly.out[0]; ++o)
                            acc += dz[o] * static_cast<double>(h16(W[o * ly.in[0] + 2 * lv + f]));
                        dx[f] = acc;
                    }
                    uint32_t e[8];
                    float w[8];
                    grid_corners(lv, q, e, w);
                    for (int c = 0; c < 8; ++c)
                        for (int f = 0; f < 2; ++f) g[ly.mlp + 2 * e[c] + f] += w[c] * dx[f];
                }
            }
            if (l == 0) break;
            // input gradient through the ReLU of the previous layer, FP16 like the GPU tile
            for (int k = 0; k < ly.in[l]; ++k) {
                double acc = 0.0;
                for (int o = 0; o < ly.out[l]; ++o) acc += dz[o] * static_cast<double>(h16(W[o * ly.in[l] + k]));
                dnext[k] = acts[l][k] > 0.0f ? static_cast<double>(h16(static_cast<float>(acc))) : 0.0;
            }
            for (int k = 0; k < ly.in[l]; ++k) dz[k] = dnext[k];
            for (int k = ly.in[l]; k < 256; ++k) dz[k] = 0.0;
        }
    }
    for (int64_t p = 0; p < ly.total; ++p) grads[p] = static_cast<float>(g[p] / loss_scale);
    return loss;
}

// Adam with L2 regularisation (learning rate lr, moments beta1/beta2, epsilon), step t >= 1.
void orc_adam(float* w, float* m, float* v, const float* grad, int64_t n, float lr, float beta1, float beta2,
              float eps, float l2, int step) {
    float c1 = 1.0f - std::pow(beta1, static_cast<float>(step));
    float c2 = 1.0f - std::pow(beta2, static_cast<float>(step));
    for (int64_t i = 0; i < n; ++i) {
        float gr = grad[i] + l2 * w[i];
        m[i] = beta1 * m[i] + (1.0f - beta1) * gr;
        v[i] = beta2 * v[i] + (1.0f - beta2) * gr * gr;
        float mh = m[i] / c1, vh = v[i] / c2;
        w[i] -= lr * mh / (std::sqrt(vh) + eps);
    }
}

}  // extern "C"
