/*
 * rtc8_nrc.hpp — the reference renderer's C++ NeuralRadianceCache interface
 * (renderer/network_interface.h:8-31, namespace rtc8) on top of the C ABI of rtc8_nrc.h, so the
 * renderer's call sites (renderer_main.cpp:1243-1247, 1310-1315, 1338-1342, 1582-1586,
 * 1603-1608, 1629-1633) compile unchanged against the GB300 cache.
 *
 * Header-only; link against librtc8_gb300.so. Same signatures and meaning as the reference:
 * the caller owns the device buffers (14-float RadianceQuery inputs, 3-float outputs), calls
 * are asynchronous on `stream`, and a non-null lossOnCPU makes train() synchronise and return
 * the batch loss. Errors throw std::runtime_error carrying nrc_last_error(), as tiny-cuda-nn
 * threw from inside the reference's implementation. PositionEncoding::HashGrid selects the
 * reference's default multiresolution hash grid + OneBlob encoding (renderer_scene.cpp:50 calls
 * initialize(HashGrid, 2, 0.01f)); PositionEncoding::TriangleWave the TriangleWave + OneBlob one.
 * initialize(const NrcConfig&) is an addition that selects any configuration of rtc8_nrc.h
 * (for example the volume encoding).
 */
#ifndef RTC8_NRC_HPP
#define RTC8_NRC_HPP

#include <cuda.h>

#include <cstdint>
#include <stdexcept>
#include <string>

#include "rtc8_nrc.h"

namespace rtc8 {

enum class PositionEncoding {
    TriangleWave,
    HashGrid,
};

class NeuralRadianceCache {
    NrcHandle* m = nullptr;

    static void check(int rc, const char* what) {
        if (rc != NRC_OK) {
            const char* msg = nrc_last_error();
            throw std::runtime_error(std::string(what) + ": " + (msg ? msg : "error"));
        }
    }

public:
    NeuralRadianceCache() = default;
    ~NeuralRadianceCache() { finalize(); }
    NeuralRadianceCache(const NeuralRadianceCache&) = delete;
    NeuralRadianceCache& operator=(const NeuralRadianceCache&) = delete;

    // network_interface.cu:50-134: encoding, hidden layers of 64, Adam learning rate.
    void initialize(PositionEncoding posEnc, uint32_t numHiddenLayers, float learningRate) {
        NrcConfig cfg;
        nrc_default_config(posEnc == PositionEncoding::HashGrid ? NRC_ENCODING_HASHGRID : NRC_ENCODING_REFERENCE,
                           &cfg);
        cfg.num_hidden_layers = static_cast<int32_t>(numHiddenLayers);
        cfg.learning_rate = learningRate;
        initialize(cfg);
    }
    void initialize(const NrcConfig& cfg) {
        finalize();
        check(nrc_create(&cfg, &m), "NeuralRadianceCache::initialize");
    }
    void finalize() {
        if (m) nrc_destroy(m);
        m = nullptr;
    }

    void infer(CUstream stream, float* inputData, uint32_t numData, float* predictionData) {
        check(nrc_infer(m, stream, inputData, numData, predictionData), "NeuralRadianceCache::infer");
    }
    void train(CUstream stream, float* inputData, float* targetData, uint32_t numData, float* lossOnCPU = nullptr) {
        check(nrc_train(m, stream, inputData, targetData, numData, lossOnCPU), "NeuralRadianceCache::train");
    }

    // The underlying handle, for the C entry points that take one (vpt_nrc_frame).
    NrcHandle* handle() const { return m; }
};

}  // namespace rtc8

#endif  // RTC8_NRC_HPP
