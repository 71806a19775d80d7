/*
 * Sky-model state generator linked against the reference's vendored Hosek-Wilkie 2013 model
 * (ext/hosek_wilkie_2013/ArHosekSkyModel.c v1.4a, compiled by oracle/build_ref.sh into
 * oracle/_ref/). For each requested (solar elevation in degrees, turbidity, ground albedo) it
 * prints, per spectral band of the renderer (16 bands, centre wavelength clamped to
 * [320, 720] nm as in analytic_sky_kernels.cu:241-242), the state the renderer uploads
 * (renderer_scene.cpp:570-592) and the solar-disc terms: the direct solar radiance at the
 * sun's elevation before limb darkening and the six interpolated limb-darkening coefficients
 * (ArHosekSkyModel.c:687-789). A negative albedo selects the renderer's per-band ramp
 * 0.5 * (1 - (i + 0.5) / 16) (renderer_scene.cpp:576). It also prints reference radiance values
 * at fixed (theta, gamma) for the first request, used to check the device port.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "ArHosekSkyModel.h"

extern double* limbDarkeningDatasets[];
/* Defined in ArHosekSkyModel.c without a header prototype. */
double arhosekskymodel_solar_radiance_internal2(ArHosekSkyModelState* state, double wavelength, double elevation,
                                                double gamma);

static const int kBands = 16;

static double center_wavelength(int i) { return 360.0 + (i + 0.5) * (830.0 - 360.0) / kBands; }

int main(int argc, char** argv) {
    int nreq = (argc - 1) / 3;
    printf("{\"entries\": [\n");
    for (int r = 0; r < nreq; ++r) {
        double elev_deg = atof(argv[1 + 3 * r]);
        double turb = atof(argv[2 + 3 * r]);
        double alb = atof(argv[3 + 3 * r]);
        double elev = elev_deg * M_PI / 180.0;
        printf("{\"elevation_deg\": %.9g, \"turbidity\": %.9g, \"albedo\": %.9g,\n \"states\": [", elev_deg, turb, alb);
        for (int b = 0; b < kBands; ++b) {
            double a = alb >= 0 ? alb : 0.5 * (1.0 - (b + 0.5) / kBands);
            ArHosekSkyModelState* st = arhosekskymodelstate_alloc_init(elev, turb, a);
            printf("%s[", b ? ",\n  " : "");
            for (int i = 0; i < 11; ++i)
                for (int j = 0; j < 9; ++j) printf("%s%.9g", (i || j) ? ", " : "", (float)st->configs[i][j]);
            for (int i = 0; i < 11; ++i) printf(", %.9g", (float)st->radiances[i]);
            for (int i = 0; i < 11; ++i) printf(", %.9g", (float)st->emission_correction_factor_sky[i]);
            printf(", %.9g]", (float)st->solar_radius);
            arhosekskymodelstate_free(st);
        }
        printf("],\n \"solar\": [");
        for (int b = 0; b < kBands; ++b) {
            double a = alb >= 0 ? alb : 0.5 * (1.0 - (b + 0.5) / kBands);
            ArHosekSkyModelState* st = arhosekskymodelstate_alloc_init(elev, turb, a);
            double wl = center_wavelength(b);
            if (wl < 320.0) wl = 320.0;
            if (wl > 720.0) wl = 720.0;
            int wl_low = (int)((wl - 320.0) / 40.0);
            double wl_frac = fmod(wl, 40.0) / 40.0;
            if (wl_low == 10) {
                wl_low = 9;
                wl_frac = 1.0;
            }
            double ld[6], ld_sum = 0.0;
            for (int i = 0; i < 6; ++i) {
                ld[i] = (1.0 - wl_frac) * limbDarkeningDatasets[wl_low][i] + wl_frac * limbDarkeningDatasets[wl_low + 1][i];
                ld_sum += ld[i];
            }
            /* At gamma = 0 the sample cosine is 1, so the darkening factor is the coefficient sum. */
            double direct = arhosekskymodel_solar_radiance_internal2(st, wl, elev, 0.0) / ld_sum;
            printf("%s[%.9g", b ? ",\n  " : "", (float)direct);
            for (int i = 0; i < 6; ++i) printf(", %.9g", (float)ld[i]);
            printf("]");
            arhosekskymodelstate_free(st);
        }
        printf("]");
        /* Direct solar radiance with limb darkening around the sun (elevation offsets d, angles
         * gamma from the sun's centre inside the disc), as the sky kernel evaluates it per texel. */
        printf(",\n \"solar_kat\": [");
        int first_s = 1;
        for (int b = 0; b < kBands; b += 5) {
            double a = alb >= 0 ? alb : 0.5 * (1.0 - (b + 0.5) / kBands);
            ArHosekSkyModelState* st = arhosekskymodelstate_alloc_init(elev, turb, a);
            double wl = center_wavelength(b);
            if (wl < 320.0) wl = 320.0;
            if (wl > 720.0) wl = 720.0;
            const double ds[3] = {-0.004, 0.0, 0.003}, gs[3] = {0.0, 0.002, 0.004};
            for (int i = 0; i < 3; ++i)
                for (int g = 0; g < 3; ++g) {
                    double e = elev + ds[i];
                    if (e <= 0.0) continue;
                    double v = arhosekskymodel_solar_radiance_internal2(st, wl, e, gs[g]);
                    printf("%s[%d, %.9g, %.9g, %.9g]", first_s ? "" : ", ", b, e, gs[g], v);
                    first_s = 0;
                }
            arhosekskymodelstate_free(st);
        }
        printf("]");
        if (r == 0) {
            /* Reference radiance at fixed view angles (theta from zenith, gamma from the sun). */
            printf(",\n \"radiance_kat\": [");
            int first = 1;
            for (int b = 0; b < kBands; b += 3) {
                double a = alb >= 0 ? alb : 0.5 * (1.0 - (b + 0.5) / kBands);
                ArHosekSkyModelState* st = arhosekskymodelstate_alloc_init(elev, turb, a);
                double wl = center_wavelength(b);
                if (wl < 320.0) wl = 320.0;
                if (wl > 720.0) wl = 720.0;
                for (int t = 0; t < 6; ++t)
                    for (int g = 0; g < 6; ++g) {
                        double theta = 0.05 + t * 0.29, gamma = 0.02 + g * 0.5;
                        double v = arhosekskymodel_radiance(st, theta, gamma, wl);
                        printf("%s[%d, %.9g, %.9g, %.9g]", first ? "" : ", ", b, theta, gamma, v);
                        first = 0;
                    }
                arhosekskymodelstate_free(st);
            }
            printf("]");
        }
        printf("}%s\n", r + 1 < nreq ? "," : "");
    }
    printf("]}\n");
    return 0;
}
