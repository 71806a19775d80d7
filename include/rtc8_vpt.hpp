/*
 * rtc8_vpt.hpp — C++ host side of the GB300 volumetric path tracer over the C ABI of rtc8_vpt.h.
 *
 * The reference drives its pipeline from renderer_main.cpp: it builds the scene (volume from an
 * .nvdb file, environment, camera), then per frame launches the path-tracing ray-generation
 * program `spp` times (numAccumFrames counting up), tone-maps the accumulation and saves
 * "%03u.png" (renderer/renderer_main.cpp:1444-1667). rtc8::VolumeRenderer owns one VptContext
 * and offers those steps as member functions; errors throw std::runtime_error with
 * vpt_last_error(). Header-only; link against librtc8_gb300.so. Not thread-safe (one host
 * thread, as the reference).
 */
#ifndef RTC8_VPT_HPP
#define RTC8_VPT_HPP

#include <cuda.h>

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "rtc8_vpt.h"

namespace rtc8 {

struct Vec3 {
    double x, y, z;
};

// Orientation quaternion (x, y, z, w) of a camera at `eye` looking at `target` with `up` for
// VptFrameParams::cam_orientation: the camera looks down its local -z axis and local +y is up
// (optix_pathtracing_kernels.cu:43-55). The rotation's columns are right, up and back; the
// quaternion comes from Shepperd's method, in double precision, normalised.
inline void look_at_quaternion(Vec3 eye, Vec3 target, Vec3 up, float q[4]) {
    auto norm = [](Vec3 v) {
        const double l = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
        return Vec3{v.x / l, v.y / l, v.z / l};
    };
    auto cross = [](Vec3 a, Vec3 b) {
        return Vec3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    };
    const Vec3 back = norm(Vec3{eye.x - target.x, eye.y - target.y, eye.z - target.z});
    const Vec3 right = norm(cross(up, back));
    const Vec3 up2 = cross(back, right);
    const double m[3][3] = {{right.x, up2.x, back.x}, {right.y, up2.y, back.y}, {right.z, up2.z, back.z}};
    const double tr = m[0][0] + m[1][1] + m[2][2];
    double x, y, z, w;
    if (tr > 0) {
        const double s = std::sqrt(tr + 1.0) * 2;
        w = 0.25 * s;
        x = (m[2][1] - m[1][2]) / s;
        y = (m[0][2] - m[2][0]) / s;
        z = (m[1][0] - m[0][1]) / s;
    } else if (m[0][0] > m[1][1] && m[0][0] > m[2][2]) {
        const double s = std::sqrt(1.0 + m[0][0] - m[1][1] - m[2][2]) * 2;
        w = (m[2][1] - m[1][2]) / s;
        x = 0.25 * s;
        y = (m[0][1] + m[1][0]) / s;
        z = (m[0][2] + m[2][0]) / s;
    } else if (m[1][1] > m[2][2]) {
        const double s = std::sqrt(1.0 + m[1][1] - m[0][0] - m[2][2]) * 2;
        w = (m[0][2] - m[2][0]) / s;
        x = (m[0][1] + m[1][0]) / s;
        y = 0.25 * s;
        z = (m[1][2] + m[2][1]) / s;
    } else {
        const double s = std::sqrt(1.0 + m[2][2] - m[0][0] - m[1][1]) * 2;
        w = (m[1][0] - m[0][1]) / s;
        x = (m[0][2] + m[2][0]) / s;
        y = (m[1][2] + m[2][1]) / s;
        z = 0.25 * s;
    }
    const double l = std::sqrt(x * x + y * y + z * z + w * w);
    q[0] = float(x / l);
    q[1] = float(y / l);
    q[2] = float(z / l);
    q[3] = float(w / l);
}

class VolumeRenderer {
    VptContext* ctx_ = nullptr;
    int32_t width_ = 0, height_ = 0;

    static void check(int rc, const char* what) {
        if (rc != VPT_OK) {
            const char* msg = vpt_last_error();
            throw std::runtime_error(std::string(what) + ": " + (msg ? msg : "error"));
        }
    }

public:
    VolumeRenderer(int32_t width, int32_t height) : width_(width), height_(height) {
        check(vpt_create(width, height, &ctx_), "vpt_create");
    }
    ~VolumeRenderer() {
        if (ctx_) vpt_destroy(ctx_);
    }
    VolumeRenderer(const VolumeRenderer&) = delete;
    VolumeRenderer& operator=(const VolumeRenderer&) = delete;

    VptContext* context() const { return ctx_; }
    int32_t width() const { return width_; }
    int32_t height() const { return height_; }

    // renderer_main.cpp:86-93: per-pixel PCG32 states from std::mt19937_64(seed).
    void seed(uint64_t seed = 591842031321323413ull) { check(vpt_seed_rng(ctx_, seed), "vpt_seed_rng"); }
    // nanovdb::io::readGrid + Scene::allocateVolumeGrid (renderer_scene.cpp:2468, 491-537).
    void load_volume(const std::string& nvdb_path, uint64_t grid_index = 0) {
        check(vpt_set_volume_nvdb_file(ctx_, nvdb_path.c_str(), grid_index), "vpt_set_volume_nvdb_file");
    }
    void set_volume_dense(const float* voxels, int32_t nx, int32_t ny, int32_t nz, float voxel_size,
                          const float origin[3]) {
        check(vpt_set_volume_dense(ctx_, voxels, nx, ny, nz, voxel_size, origin), "vpt_set_volume_dense");
    }
    // Image-based environment (rows = polar angle from +y) and its importance map.
    void set_environment(const float* rgb, int32_t width, int32_t height) {
        check(vpt_set_environment_rgb(ctx_, rgb, width, height), "vpt_set_environment_rgb");
    }
    void set_constant_environment(float r, float g, float b, int32_t width = 64, int32_t height = 32) {
        std::vector<float> img(static_cast<size_t>(width) * height * 3);
        for (size_t i = 0; i < img.size(); i += 3) {
            img[i] = r;
            img[i + 1] = g;
            img[i + 2] = b;
        }
        set_environment(img.data(), width, height);
    }
    void set_frame(const VptFrameParams& f) { check(vpt_set_frame_params(ctx_, &f), "vpt_set_frame_params"); }
    void set_tracker(int32_t kind) { check(vpt_set_tracker(ctx_, kind, 0, 0, 0), "vpt_set_tracker"); }

    // pathTrace raygen launched for `spp` samples per pixel (renderer_main.cpp:1617-1644).
    void path_trace(CUstream stream, uint32_t spp) { check(vpt_launch_plain(ctx_, stream, spp), "vpt_launch_plain"); }
    // One radiance-cache frame (renderer_main.cpp:1553-1637) with the cache handle of rtc8_nrc.h
    // (rtc8::NeuralRadianceCache::handle()).
    void nrc_frame(void* nrc_handle, CUstream stream, uint32_t train_iterations, uint32_t spp, bool new_sequence) {
        check(vpt_nrc_frame(ctx_, nrc_handle, stream, train_iterations, spp, new_sequence ? 1 : 0), "vpt_nrc_frame");
    }
    void synchronize(CUstream stream) { check(vpt_synchronize(ctx_, stream), "vpt_synchronize"); }
    void reset_accumulation() { check(vpt_reset_accumulation(ctx_), "vpt_reset_accumulation"); }

    // applyToneMap + saveImage's sRGB 8-bit conversion: the frame of "%03u.png".
    std::vector<uint32_t> image_rgba8(float brightness = 1.0f, uint32_t flags = VPT_SDR_SRGB) {
        std::vector<uint32_t> out(static_cast<size_t>(width_) * height_);
        check(vpt_download_image_rgba8(ctx_, brightness, flags, out.data()), "vpt_download_image_rgba8");
        return out;
    }
    std::vector<float> mean_rgb() {
        std::vector<float> out(static_cast<size_t>(width_) * height_ * 3);
        check(vpt_download_mean(ctx_, out.data()), "vpt_download_mean");
        return out;
    }
    uint32_t device_errors() { return vpt_get_device_errors(ctx_); }
};

}  // namespace rtc8

#endif  // RTC8_VPT_HPP
