/*
 * A plain C caller of the engine's C ABI (include/fargocpt_gb300.h), the way
 * a host program other than Python drives it: create an engine from an
 * fgpu_params block, upload FargoCPT-layout fields, set the bodies, run the
 * start-up calls and CFL-limited Euler steps, read the disk force and the
 * fields back.  Used by tests/test_gpu_abi_client.py, which writes the inputs
 * and checks the outputs against the oracle.
 *
 *   abi_client <dir> <steps>
 *
 * reads <dir>/params.bin (one fgpu_params), radii.bin (nrad + 2 doubles),
 * bodies.bin (fgpu_body records), SIGMA.bin, V_RADIAL.bin, V_AZIMUTHAL.bin,
 * ENERGY.bin (raw FP64 rows); writes <dir>/out_<field>.bin, out_dt.bin (the
 * dt of every step) and out_force.bin (2 doubles per body).
 */
#include "fargocpt_gb300.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static char g_dir[4096];

static void *read_file(const char *name, size_t *bytes)
{
    char path[4200];
    snprintf(path, sizeof path, "%s/%s", g_dir, name);
    FILE *f = fopen(path, "rb");
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path);
        exit(2);
    }
    fseek(f, 0, SEEK_END);
    const long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    void *buf = malloc((size_t)n > 0 ? (size_t)n : 1);
    if (!buf || fread(buf, 1, (size_t)n, f) != (size_t)n) {
        fprintf(stderr, "cannot read %s\n", path);
        exit(2);
    }
    fclose(f);
    *bytes = (size_t)n;
    return buf;
}

static void write_file(const char *name, const void *data, size_t bytes)
{
    char path[4200];
    snprintf(path, sizeof path, "%s/%s", g_dir, name);
    FILE *f = fopen(path, "wb");
    if (!f || fwrite(data, 1, bytes, f) != bytes) {
        fprintf(stderr, "cannot write %s\n", path);
        exit(2);
    }
    fclose(f);
}

static fgpu_engine *g_eng;

static void check(int rc, const char *what)
{
    if (rc != FGPU_OK) {
        fprintf(stderr, "%s failed: %d (%s)\n", what, rc,
                g_eng ? fgpu_last_error(g_eng) : "no engine");
        exit(1);
    }
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s <dir> <steps>\n", argv[0]);
        return 2;
    }
    snprintf(g_dir, sizeof g_dir, "%s", argv[1]);
    const int steps = atoi(argv[2]);
    size_t n;
    fgpu_params *p = (fgpu_params *)read_file("params.bin", &n);
    if (n != sizeof(fgpu_params)) {
        fprintf(stderr, "params.bin holds %zu bytes, fgpu_params is %zu\n", n, sizeof(fgpu_params));
        return 2;
    }
    double *radii = (double *)read_file("radii.bin", &n);
    fgpu_body *bodies = (fgpu_body *)read_file("bodies.bin", &n);
    const int nbodies = (int)(n / sizeof(fgpu_body));
    const int nr = p->nrad, nz = p->naz;

    check(fgpu_create(p, radii, &g_eng), "fgpu_create");
    static const struct {
        const char *file;
        int field, ref, rows_extra;
    } fields[4] = {{"SIGMA.bin", FGPU_SIGMA, FGPU_SIGMA0, 0},
                   {"V_RADIAL.bin", FGPU_V_RADIAL, FGPU_V_RADIAL0, 1},
                   {"V_AZIMUTHAL.bin", FGPU_V_AZIMUTHAL, FGPU_V_AZIMUTHAL0, 0},
                   {"ENERGY.bin", FGPU_ENERGY, FGPU_ENERGY0, 0}};
    for (int k = 0; k < 4; ++k) {
        double *a = (double *)read_file(fields[k].file, &n);
        const int rows = nr + fields[k].rows_extra;
        if (n != (size_t)rows * nz * sizeof(double)) {
            fprintf(stderr, "%s has the wrong size\n", fields[k].file);
            return 2;
        }
        check(fgpu_upload_field(g_eng, fields[k].field, a, rows, nz), "fgpu_upload_field");
        check(fgpu_upload_field(g_eng, fields[k].ref, a, rows, nz), "fgpu_upload_field");
        free(a);
    }
    check(fgpu_set_bodies(g_eng, nbodies, bodies, 0.0, 0.0, 0.0), "fgpu_set_bodies");
    check(fgpu_init_euler(g_eng, 0.0), "fgpu_init_euler");
    check(fgpu_apply_boundary_condition(g_eng, 0.0, 0.0, 0), "fgpu_apply_boundary_condition");

    double *dts = (double *)calloc((size_t)steps > 0 ? (size_t)steps : 1, sizeof(double));
    double t = 0.0;
    for (int s = 0; s < steps; ++s) {
        double dt;
        check(fgpu_condition_cfl(g_eng, &dt), "fgpu_condition_cfl");
        check(fgpu_step_euler(g_eng, dt, t), "fgpu_step_euler");
        dts[s] = dt;
        t += dt;
    }
    double *force = (double *)calloc(2 * (size_t)nbodies, sizeof(double));
    check(fgpu_disk_on_nbody_accel(g_eng, force), "fgpu_disk_on_nbody_accel");
    for (int k = 0; k < 4; ++k) {
        const int rows = nr + fields[k].rows_extra;
        double *a = (double *)malloc((size_t)rows * nz * sizeof(double));
        check(fgpu_download_field(g_eng, fields[k].field, a, rows, nz), "fgpu_download_field");
        char name[64];
        snprintf(name, sizeof name, "out_%s", fields[k].file);
        write_file(name, a, (size_t)rows * nz * sizeof(double));
        free(a);
    }
    write_file("out_dt.bin", dts, (size_t)steps * sizeof(double));
    write_file("out_force.bin", force, 2 * (size_t)nbodies * sizeof(double));
    check(fgpu_destroy(g_eng), "fgpu_destroy");
    free(dts);
    free(force);
    free(p);
    free(radii);
    free(bodies);
    printf("abi_client: %d steps, t = %.17g\n", steps, t);
    return 0;
}
