/*
 * field_dump.c -- a binary field writer with the signature of the reference's
 * VTK writer (src/vtksave.c:29-30), compiled into a second build of the
 * reference's CUDA program in place of src/vtksave.c.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build.py (build_reference_dump) stages
 * the reference's sources unmodified into oracle/_ref/src_dump, except that
 * this file takes the name vtksave.c there, and compiles src/main.cu from that
 * directory into oracle/_ref/lbm_ref_cuda_dump (src/Makefile's -O3
 * -use_fast_math) and oracle/_ref/lbm_ref_cuda_exact_dump (-O3).  src/main.cu
 * calls vtkSave at its output points (src/main.cu:302, :472, :490, :607, :636)
 * after copying phi, rho, ux, uy, uz back from the device, so these builds
 * hand the reference's own GPU fields to the parity tests at full float
 * precision; the reference's writer prints them with "%f"
 * (src/vtksave.c:60-138), six decimals, too coarse for velocities ~1e-5.
 *
 * It is part of the reference's single translation unit (src/main.cu:57
 * includes vtksave.c by name), so it reads the reference's globals RELAX, step,
 * NX_h, NY_h, NZ_h and gridId_h (src/constants.h:62-65, src/gridid.c:27-30).
 *
 * Nothing is written unless the environment variable LBM_DUMP_STEPS lists the
 * call's step (comma-separated numbers, or "all").  The file
 * <relax|data>_<step>.f32 in the working directory then holds five blocks of
 * NX_h * NY_h * (NZ_h - 2) floats, x fastest, over the interior planes
 * k = 1 .. NZ_h - 2: phi, rho, ux, uy, uz.  "relax" marks the calls made while
 * the reference's RELAX flag is set (the initial state and the relaxation loop).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static int field_dump_wanted(int at_step)
{
    const char *list = getenv("LBM_DUMP_STEPS");
    if (!list || !*list) return 0;
    if (strcmp(list, "all") == 0) return 1;
    const char *p = list;
    while (*p) {
        char *end = NULL;
        const long v = strtol(p, &end, 10);
        if (end == p) return 0;
        if (v == at_step) return 1;
        p = end;
        while (*p == ',' || *p == ' ') p++;
    }
    return 0;
}

int vtkSave(int *nb_east, int *nb_west, int *nb_north, int *nb_south, float *phi, float *rho, float *ux,
            float *uy, float *uz)
{
    (void)nb_east;
    (void)nb_west;
    (void)nb_north;
    (void)nb_south;
    if (!field_dump_wanted(step)) return 0;
    char name[64];
    snprintf(name, sizeof(name), "%s_%07d.f32", RELAX == 0 ? "data" : "relax", step);
    FILE *fp = fopen(name, "wb");
    if (!fp) {
        fprintf(stderr, "field_dump: cannot open %s\n", name);
        return 1;
    }
    float *const fields[5] = {phi, rho, ux, uy, uz};
    const size_t plane = (size_t)NX_h * (size_t)NY_h;
    int ok = 1;
    for (int a = 0; a < 5 && ok; a++)
        for (int k = 1; k < NZ_h - 1 && ok; k++)
            ok = fwrite(fields[a] + gridId_h(0, 0, k), sizeof(float), plane, fp) == plane;
    fclose(fp);
    if (!ok) fprintf(stderr, "field_dump: short write to %s\n", name);
    return ok ? 0 : 1;
}
