/*
 * rtc8_nrc.h — C ABI of the GB300 neural radiance cache (fused FP16 MLP on tcgen05).
 *
 * Replaces rtc8::NeuralRadianceCache (renderer/network_interface.h:8-31) and its tiny-cuda-nn
 * implementation (renderer/network_interface.cu:50-192):
 *   initialize(PositionEncoding, numHiddenLayers, learningRate) -> nrc_create
 *   finalize()                                                 -> nrc_destroy
 *   infer(stream, inputData, numData, predictionData)          -> nrc_infer
 *   train(stream, inputData, targetData, numData, lossOnCPU)   -> nrc_train
 * Conventions kept from the reference: the caller owns every device buffer; inputs are AoS
 * RadianceQuery records of 14 floats (renderer_shared.h:46-54: position[3] in [0,1]^3 of the
 * world box, normal_phi, normal_theta, vOut_phi, vOut_theta (radians, as written by
 * createRadianceQuery, optix_pathtracing_kernels.cu:14-29), roughness, diffuse[3],
 * specular[3]); outputs are 3 floats per record; calls are asynchronous on `stream` (a
 * cudaStream_t passed as void*); a non-null loss pointer makes nrc_train synchronise and return
 * the batch loss. Differences: any n is accepted (the reference asserts n % 128 == 0 in debug
 * builds only, network_interface.cu:178, 186); errors are status codes, not exceptions.
 */
#ifndef RTC8_NRC_H
#define RTC8_NRC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NRC_OK 0
#define NRC_ERR_INVALID_ARGUMENT (-1)
#define NRC_ERR_CUDA (-2)
#define NRC_ERR_DEVICE (-5)   /* a bounded device-side wait gave up; the context stays usable */

/* Input encodings. */
#define NRC_ENCODING_REFERENCE 0   /* TriangleWave(12) on position, OneBlob(4) on the 5 angle /
                                      roughness dims (angles normalised to [0,1]), identity on
                                      the 6 reflectance dims: network_interface.cu:108-129 */
#define NRC_ENCODING_VOLUME 1      /* sin/cos 12 frequencies on position, OneBlob(32) on the
                                      outgoing direction (theta, phi), identity on the local
                                      density (roughness slot) and albedo (diffuse.r) */
#define NRC_ENCODING_HASHGRID 2    /* the reference's default (network_interface.cu:99-122):
                                      multiresolution hash grid on position (16 levels x 2
                                      features, 2^15 entries per level, base resolution 16,
                                      per-level scale 2; positions clamped to [0,1]^3), then
                                      OneBlob(4) and identity as NRC_ENCODING_REFERENCE. The
                                      tables are trained parameters: they follow the MLP
                                      matrices in nrc_get_params / nrc_set_params /
                                      nrc_get_gradients (level by level, entry by entry, two
                                      features per entry) */

#define NRC_OUTPUT_NONE 0          /* reference: output_activation None */
#define NRC_OUTPUT_EXP 1

typedef struct NrcConfig {
    int32_t encoding;              /* NRC_ENCODING_* */
    int32_t num_hidden_layers;     /* 64 neurons each; reference 2 (renderer_scene.cpp:50) */
    int32_t output_activation;     /* NRC_OUTPUT_* */
    float learning_rate;           /* Adam (network_interface.cu:88-98) */
    float beta1, beta2, epsilon, l2_reg;
    float ema_decay;               /* EMA of the weights used for inference; 0 = off */
    float loss_scale;              /* FP16 gradient scaling */
    uint32_t seed;                 /* weight initialisation */
} NrcConfig;

typedef struct NrcHandle NrcHandle;

/* Fills `cfg` with the reference's settings for the given encoding. */
void nrc_default_config(int32_t encoding, NrcConfig* cfg);
int nrc_create(const NrcConfig* cfg, NrcHandle** out);
int nrc_destroy(NrcHandle* h);
const char* nrc_last_error(void);

/* Network inference: out[3*i..] = MLP(encode(in[14*i..])), i < n. */
int nrc_infer(NrcHandle* h, void* stream, const float* in, uint32_t n, float* out);
/* Inference on a device-resident count (*dev_n <= n_max), so a pipeline needs no host sync. */
int nrc_infer_device_count(NrcHandle* h, void* stream, const float* in, const uint32_t* dev_n, uint32_t n_max,
                           float* out);
/* Inference on the records listed in idx[0 .. *dev_n) (*dev_n <= n_max, device-resident): record
 * k = idx[i] reads in[14*k..] and writes out[3*k..]; the other records of `out` are left as they
 * are. For query buffers where only some slots hold a query (a render pass lists the slots its
 * paths ended with a cache query in). */
int nrc_infer_indexed(NrcHandle* h, void* stream, const float* in, const uint32_t* idx, const uint32_t* dev_n,
                      uint32_t n_max, float* out);
/* One training step on n records: forward, relative-L2-luminance loss, backward, Adam. */
int nrc_train(NrcHandle* h, void* stream, const float* in, const float* target, uint32_t n, float* loss_or_null);

/* Parameter access (FP32 master weights, layer by layer, each layer row-major
 * [out][in] with the padded sizes reported by nrc_get_layout; with NRC_ENCODING_HASHGRID the
 * hash-grid tables follow the last layer, and total_params counts them). */
int nrc_get_layout(NrcHandle* h, int32_t* num_layers, int32_t* in_dims, int32_t* out_dims, int64_t* total_params);
int nrc_get_params(NrcHandle* h, float* host_params);
int nrc_set_params(NrcHandle* h, const float* host_params);
/* Gradient of the last nrc_train call (unscaled, same layout as the parameters). */
int nrc_get_gradients(NrcHandle* h, float* host_grads);
/* Encoded, padded network input of n records (n x in_dims[0] FP32), for testing the encoders. */
int nrc_encode(NrcHandle* h, void* stream, const float* in, uint32_t n, float* out);
uint64_t nrc_step_count(NrcHandle* h);
/* Error bits of bounded device-side waits (tensor-core completion) since the last call; 0 = ok. */
uint32_t nrc_device_errors(NrcHandle* h);

/* Tensor-core self test: D = A * B^T for A (128 x 64) and B (64 x 64) given as FP32 host arrays
 * (rounded to FP16), with the operands staged in shared memory K-major (0) or MN-major (1);
 * writes D (128 x 64, FP32) to host memory. Checks the shared-memory descriptor layouts the
 * MLP kernels rely on. */
int nrc_selftest_mma(const float* a, const float* b, int32_t a_mn_major, int32_t b_mn_major, float* d);
/* Tensor-core issue-rate probe: one thread issues `count` (rounded up to a multiple of 4, at most
 * 65536) back-to-back tcgen05 MMAs of M = 128, N = `n` (a multiple of 16 in [16, 256]), K = 16,
 * FP16 operands in shared memory, FP32 accumulators in tensor memory, on one SM; writes the SM
 * clock cycles per MMA from the first issue to the completion of the last. It measures the rate
 * the MLP kernels' MMA shapes can reach (their hidden layers are N = 64). */
int nrc_selftest_mma_rate(int32_t n, uint32_t count, double* cycles_per_mma);

#ifdef __cplusplus
}
#endif

#endif /* RTC8_NRC_H */
