// Known-answer generator built from the reference's own common/basic_types.{h,cpp} (host code
// only, compiled by oracle/build_ref.sh into oracle/_ref/). Prints JSON with the outputs of the
// reference's math helpers on fixed inputs; tests/golden/make_golden.py stores them as fixtures.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>

#include "basic_types.h"

using namespace rtc8;

static void print_floats(const char* name, const float* v, int n, bool last = false) {
    std::printf("\"%s\": [", name);
    for (int i = 0; i < n; ++i) std::printf("%s%.9g", i ? ", " : "", v[i]);
    std::printf("]%s\n", last ? "" : ",");
}

int main() {
    std::mt19937 gen(12345);
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    const int N = 64;
    float vin[3 * N], polar[2 * N], frames[6 * N], fromp[3 * N], pin[2 * N];
    for (int i = 0; i < N; ++i) {
        Vector3D v(u(gen), u(gen), u(gen));
        if (i == 0) v = Vector3D(0, 0, 1);
        if (i == 1) v = Vector3D(0, 0, -1);
        if (i == 2) v = Vector3D(0, 1, 0);
        v = normalize(v);
        vin[3 * i] = v.x;
        vin[3 * i + 1] = v.y;
        vin[3 * i + 2] = v.z;
        float theta, phi;
        v.toPolarYUp(&theta, &phi);
        polar[2 * i] = theta;
        polar[2 * i + 1] = phi;
        Vector3D t, b;
        v.makeCoordinateSystem(&t, &b);
        frames[6 * i] = t.x;
        frames[6 * i + 1] = t.y;
        frames[6 * i + 2] = t.z;
        frames[6 * i + 3] = b.x;
        frames[6 * i + 4] = b.y;
        frames[6 * i + 5] = b.z;
        float ph = (u(gen) + 1.0f) * 3.14159265f, th = (u(gen) + 1.0f) * 0.5f * 3.14159265f;
        pin[2 * i] = ph;
        pin[2 * i + 1] = th;
        Vector3D w = Vector3D::fromPolarYUp(ph, th);
        fromp[3 * i] = w.x;
        fromp[3 * i + 1] = w.y;
        fromp[3 * i + 2] = w.z;
    }
    float qin[4 * 8], mats[9 * 8];
    for (int i = 0; i < 8; ++i) {
        Quaternion q(u(gen), u(gen), u(gen), u(gen));
        q = normalize(q);
        qin[4 * i] = q.x;
        qin[4 * i + 1] = q.y;
        qin[4 * i + 2] = q.z;
        qin[4 * i + 3] = q.w;
        Matrix3x3 m = q.toMatrix3x3();
        float vals[9] = {m.m00, m.m10, m.m20, m.m01, m.m11, m.m21, m.m02, m.m12, m.m22};
        for (int k = 0; k < 9; ++k) mats[9 * i + k] = vals[k];
    }
    float cmf[65];
    computeDiscretizedXyzCmfs(16, cmf + 48, cmf, cmf + 16, cmf + 32, cmf + 64);
    float lum_in[3] = {0.25f, 0.5f, 0.75f};
    float lum = RGBSpectrum(lum_in[0], lum_in[1], lum_in[2]).luminance();

    // sRGB_gamma_s (basic_types.h:3181-3188) on fixed inputs, and the output path of the
    // headless loop: applyToneMap (renderer/gpu_kernels/post_process_kernels.cu:10-41, device code
    // there, evaluated here on the host with the same RGBSpectrum and std functions) followed by
    // saveImage's 8-bit conversion (common/common_host.cpp:517-568, applyToneMap off, sRGB on).
    const int NS = 40;
    float srgb_in[NS], srgb_out[NS];
    for (int i = 0; i < NS; ++i) {
        float v = 0.5f * (u(gen) + 1.0f) * 1.25f;
        if (i == 0) v = 0.0f;
        if (i == 1) v = 0.0031308f;
        if (i == 2) v = std::nextafter(0.0031308f, 1.0f);
        if (i == 3) v = 1.0f;
        if (i == 4) v = 1e-4f;
        srgb_in[i] = v;
        srgb_out[i] = sRGB_gamma_s(v);
    }
    const int NT = 96;
    float tm_in[3 * NT], tm_out[3 * NT], tm_bytes[3 * NT];
    for (int i = 0; i < NT; ++i) {
        RGBSpectrum c((u(gen) + 1.0f) * 1.5f, (u(gen) + 1.0f) * 1.5f, (u(gen) + 1.0f) * 1.5f);
        if (i == 0) c = RGBSpectrum(0.0f, 0.0f, 0.0f);
        if (i == 1) c = RGBSpectrum(0.0f, 0.25f, 0.0f);
        if (i == 2) c = RGBSpectrum(40.0f, 0.001f, 0.5f);
        tm_in[3 * i] = c.r;
        tm_in[3 * i + 1] = c.g;
        tm_in[3 * i + 2] = c.b;
        constexpr float gamma = 1.0f / 0.6f;
        c.r = std::pow(c.r, gamma);
        c.g = std::pow(c.g, gamma);
        c.b = std::pow(c.b, gamma);
        float lum = c.luminance();
        if (lum > 0.0f) {
            float lumT = 1 - std::exp(-1.0f * lum);
            c *= lumT / lum;
        }
        tm_out[3 * i] = c.r;
        tm_out[3 * i + 1] = c.g;
        tm_out[3 * i + 2] = c.b;
        RGBSpectrum v = c;
        if (v.hasNegative()) v = max(v, RGBSpectrum::Zero());
        v = sRGB_gamma(v);
        tm_bytes[3 * i] = static_cast<float>(std::min<uint32_t>(static_cast<uint32_t>(v.r * 255), 255));
        tm_bytes[3 * i + 1] = static_cast<float>(std::min<uint32_t>(static_cast<uint32_t>(v.g * 255), 255));
        tm_bytes[3 * i + 2] = static_cast<float>(std::min<uint32_t>(static_cast<uint32_t>(v.b * 255), 255));
    }

    std::printf("{\n");
    print_floats("dirs", vin, 3 * N);
    print_floats("polar_yup_theta_phi", polar, 2 * N);
    print_floats("coordinate_system_tb", frames, 6 * N);
    print_floats("from_polar_in_phi_theta", pin, 2 * N);
    print_floats("from_polar_yup", fromp, 3 * N);
    print_floats("quats", qin, 32);
    print_floats("quat_matrices_colmajor", mats, 72);
    print_floats("cmf_xs_ys_zs_centers_integral", cmf, 65);
    print_floats("luminance_of_0.25_0.5_0.75", &lum, 1);
    print_floats("srgb_gamma_in", srgb_in, NS);
    print_floats("srgb_gamma_out", srgb_out, NS);
    print_floats("tonemap_mean_rgb", tm_in, 3 * NT);
    print_floats("tonemap_out_rgb", tm_out, 3 * NT);
    print_floats("tonemap_srgb_bytes", tm_bytes, 3 * NT, true);
    std::printf("}\n");
    return 0;
}
