/*
 * Writes the coefficient tables of the Hosek-Wilkie 2013 spectral sky model (v1.4a, the version
 * the reference vendors in ext/hosek_wilkie_2013) to a binary file, so that rtc8_gb300/sky.py can
 * compute the per-band model states for any solar elevation, turbidity and ground albedo the way
 * the reference does every frame (renderer/renderer_scene.cpp:555-592 ->
 * arhosekskymodelstate_alloc_init). rtc8_gb300/build.py compiles it against the model's source in
 * the reference checkout and writes rtc8_gb300/data/hosek_tables.bin (generated, not committed).
 *
 * Layout: the ASCII tag "HOSEK1", two padding bytes, then float64 arrays, channel by channel for
 * the 11 channels 320, 360, ..., 720 nm:
 *   configuration datasets  11 x 1080  (albedo 0/1 x turbidity 1..10 x 6 Bezier points x 9)
 *   radiance datasets       11 x 120   (albedo 0/1 x turbidity 1..10 x 6 Bezier points)
 *   solar datasets          11 x 1800  (turbidity 1..10 x 45 pieces x 4 coefficients)
 *   limb darkening          11 x 6
 */
#include <stdio.h>

extern double* datasets[];
extern double* datasetsRad[];
extern double* solarDatasets[];
extern double* limbDarkeningDatasets[];

static int put(FILE* f, const double* p, size_t n) { return fwrite(p, sizeof(double), n, f) == n ? 0 : 1; }

int main(int argc, char** argv) {
    if (argc != 2) {
        fprintf(stderr, "usage: hosek_tables_gen <out.bin>\n");
        return 2;
    }
    FILE* f = fopen(argv[1], "wb");
    if (!f) return 1;
    int err = fwrite("HOSEK1\0\0", 1, 8, f) != 8;
    for (int wl = 0; wl < 11; ++wl) err |= put(f, datasets[wl], 1080);
    for (int wl = 0; wl < 11; ++wl) err |= put(f, datasetsRad[wl], 120);
    for (int wl = 0; wl < 11; ++wl) err |= put(f, solarDatasets[wl], 1800);
    for (int wl = 0; wl < 11; ++wl) err |= put(f, limbDarkeningDatasets[wl], 6);
    err |= fclose(f) != 0;
    return err;
}
