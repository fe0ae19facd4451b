/*
 * porelb_main.c - drop-in replacement of the reference solver executable
 * (porelb.c:402-443, "porelb.x it_max").
 *
 * Same argv, same input (V.bin in the working directory), same dump names
 * and schedule: part_%03d_%07d.bin for every rank of the table after step
 * it whenever it % 1000 == 0 (so the dump tagged it holds it+1 steps), and a
 * final dump tagged it_max.  All rank slabs run on one GPU; a table written
 * for num_p ranks is run with the semantics of `mpirun -np num_p`.
 *
 * Extra options (the reference hard-codes them in init_para, porelb.c:83-94):
 *   --tau T  --force F  --precision fp64_exact|fp64|fp32|fp16dev|bf16dev
 *   --save-every S  --vbin PATH  --outdir DIR  --device D  --single-rank
 * Exit codes follow the reference: -1 open error, -5 read error, -6 density
 * guard, -10 usage; -4 for a CUDA error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "porelb_gpu.h"

static double now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int parse_precision(const char *s)
{
    if (!strcmp(s, "fp64_exact")) return PLB_FP64_EXACT;
    if (!strcmp(s, "fp64")) return PLB_FP64;
    if (!strcmp(s, "fp32")) return PLB_FP32;
    if (!strcmp(s, "fp16dev")) return PLB_FP16DEV;
    if (!strcmp(s, "bf16dev")) return PLB_BF16DEV;
    if (!strcmp(s, "fp64_fma")) return PLB_FP64_FMA;
    return -1;
}

int main(int argc, char **argv)
{
    plb_params prm;
    plb_default_params(&prm);
    const char *vbin = "V.bin", *outdir = NULL;
    int it_max = -1, save_every = 1000;
    for (int a = 1; a < argc; a++) {
        if (!strcmp(argv[a], "--tau") && a + 1 < argc) prm.tau = atof(argv[++a]);
        else if (!strcmp(argv[a], "--force") && a + 1 < argc) prm.force_x = atof(argv[++a]);
        else if (!strcmp(argv[a], "--precision") && a + 1 < argc) prm.precision = parse_precision(argv[++a]);
        else if (!strcmp(argv[a], "--save-every") && a + 1 < argc) save_every = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--vbin") && a + 1 < argc) vbin = argv[++a];
        else if (!strcmp(argv[a], "--outdir") && a + 1 < argc) outdir = argv[++a];
        else if (!strcmp(argv[a], "--device") && a + 1 < argc) prm.device = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--single-rank")) prm.halo = PLB_HALO_SINGLE;
        else if (it_max < 0 && argv[a][0] != '-') it_max = atoi(argv[a]);
        else {
            fprintf(stderr, ">>> Error argc, usage ./porelb.x it_max [options]\n");
            return -10;
        }
    }
    if (it_max < 0 || prm.precision < 0 || save_every <= 0) {
        fprintf(stderr, ">>> Error argc, usage ./porelb.x it_max [options]\n");
        return -10;
    }
    int num_f, num_p, nx, ny, nz;
    if (plb_read_vbin_header(vbin, &num_f, &num_p, &nx, &ny, &nz) != PLB_OK) {
        fprintf(stderr, "Node map file openning error!\n");
        return -1;
    }
    printf("[0]>>> Total num of fluid  nodes = %d\n", num_f);
    plb_node_info *V = (plb_node_info *)malloc(sizeof(plb_node_info) * (size_t)(num_f ? num_f : 1));
    int *vs = (int *)malloc(sizeof(int) * (size_t)num_p);
    if (!V || !vs) {
        fprintf(stderr, "0 >>> Error calloc memory for V \n");
        return -4;
    }
    if (plb_read_vbin(vbin, V, vs) != PLB_OK) {
        fprintf(stderr, "0 >>> Error read V \n");
        return -5;
    }
    int rc = plb_check_table(V, num_f, nx, ny, nz, num_p, vs);
    if (rc != PLB_OK) {
        fprintf(stderr, "0 >>> Check V, bound error!\n");
        return -3;
    }
    plb_sim *sim = NULL;
    rc = plb_create(V, num_f, nx, ny, nz, num_p, vs, &prm, &sim);
    if (rc != PLB_OK) {
        fprintf(stderr, ">>> plb_create: %s\n", plb_status_string(rc));
        return rc == PLB_ERR_TABLE ? -3 : -4;
    }
    free(V);
    rc = plb_init_equilibrium(sim);
    const double t1 = now();
    int it = 0;
    while (rc == PLB_OK && it < it_max) {
        /* next iteration whose end triggers a dump (it % save_every == 0) */
        int d = ((it + save_every - 1) / save_every) * save_every;
        int last = d < it_max ? d : it_max - 1;
        rc = plb_step(sim, it, last - it + 1);
        if (rc != PLB_OK) break;
        printf(">>> Step : %20d \n", last);
        if (last == d) rc = plb_save_parts(sim, outdir, d);
        it = last + 1;
    }
    if (rc == PLB_ERR_DENSITY) {
        int bit, bnode, x, y, z;
        double r;
        plb_last_error(sim, &bit, &bnode, &x, &y, &z, &r);
        fprintf(stderr, "0 >>> at %d (%d, %d, %d),  Macro denstity  = %g , < 0.5 ! (step %d)\n",
                bnode, x, y, z, r, bit);
        plb_destroy(sim);
        return -6;
    }
    if (rc != PLB_OK) {
        fprintf(stderr, ">>> %s\n", plb_status_string(rc));
        plb_destroy(sim);
        return rc == PLB_ERR_IO ? -3 : -4;
    }
    printf("Elapsed time is %f\n", now() - t1);
    rc = plb_save_parts(sim, outdir, it_max);
    plb_destroy(sim);
    if (rc != PLB_OK) {
        fprintf(stderr, "Macro binary file open error!\n");
        return -3;
    }
    return 0;
}
