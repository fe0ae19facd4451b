/*
 * ref_harness.c - drives the reference solver, compiled from the reference's
 * own porelb.c (included below from the reference tree), for the test oracle.
 * Ranks of an mpirun run are threads over the in-process MPI shim.
 * TEST INFRASTRUCTURE ONLY; built by oracle/Makefile into oracle/_ref/.
 *
 * ref_run() follows main (porelb.c:402-443) call for call, with tau and the
 * body force overridden after init_para (they are hard-coded there,
 * porelb.c:87,91) and the per-step progress printf left out.
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define main porelb_reference_main
#include "porelb.c"
#undef main

typedef struct {
    int rank, it_max, save, save_every;
    double tau, force;
    int set_tau, set_force;
    const int *start;
    double *f0, *f1, *mac;
    int num_f;
    double elapsed;
} ref_job;

static void *ref_rank_main(void *arg)
{
    ref_job *J = (ref_job *)arg;
    shim_set_rank(J->rank);
    SIMULATION sim;
    memset(&sim, 0, sizeof(sim));
    sim.it_max = J->it_max;
    MPI_Comm_rank(MPI_COMM_WORLD, &sim.pid);
    MPI_Comm_size(MPI_COMM_WORLD, &sim.num_p);
    alloc_memory(&sim);
    check_V(&sim);
    init_para(&sim);
    if (J->set_tau) {
        sim.tau = J->tau;
        sim.omega = 1.0 / sim.tau;
        sim.nu = 1.0 / 3.0 * (sim.tau - 0.5);
    }
    if (J->set_force) sim.Xforce = J->force;
    if (J->save_every > 0) sim.it_save_data = J->save_every;
    build_send_recv_info(&sim);
    init_dist_macro(&sim);
    double t1 = MPI_Wtime();
    for (sim.it = 0; sim.it < sim.it_max; sim.it++) {
        update_send_dist(&sim);
        send_recv(&sim);
        stream_inner_nodes(&sim);
        MPI_Waitall(sim.N_p, sim.send_request, MPI_STATUS_IGNORE);
        MPI_Waitall(sim.N_p, sim.recv_request, MPI_STATUS_IGNORE);
        update_recv_dist(&sim);
        collision(&sim);
        if (J->save && sim.it % sim.it_save_data == 0) save_data(&sim);
    }
    J->elapsed = MPI_Wtime() - t1;
    if (J->save) save_data(&sim);
    const size_t off = (size_t)J->start[sim.pid];
    if (J->f0) memcpy(J->f0 + off * Q, sim.f0, sizeof(double) * (size_t)sim.N * Q);
    if (J->f1) memcpy(J->f1 + off * Q, sim.f1, sizeof(double) * (size_t)sim.N * Q);
    if (J->mac) {
        const size_t n = (size_t)J->num_f;
        memcpy(J->mac + off, sim.Rho, sizeof(double) * (size_t)sim.N);
        memcpy(J->mac + n + off, sim.Ux, sizeof(double) * (size_t)sim.N);
        memcpy(J->mac + 2 * n + off, sim.Uy, sizeof(double) * (size_t)sim.N);
        memcpy(J->mac + 3 * n + off, sim.Uz, sizeof(double) * (size_t)sim.N);
    }
    free_memory(&sim);
    return NULL;
}

/* Run the reference on V.bin in workdir with num_ranks thread-ranks.
 * tau/force NaN keep the reference's hard-coded values.  f0/f1 receive the
 * global AoS arrays (V.bin order), mac receives rho|ux|uy|uz; any may be
 * NULL.  save != 0 writes the part files into workdir as main does.
 * Returns 0, or -1 when V.bin cannot be read. */
int ref_run(const char *workdir, int num_ranks, int it_max, double tau,
            double force, int save, int save_every, double *f0, double *f1,
            double *mac, double *elapsed)
{
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) return -1;
    if (chdir(workdir) != 0) return -1;
    FILE *fp = fopen("V.bin", "rb");
    if (!fp) { if (chdir(cwd)) {} return -1; }
    int hdr[5];
    if (fread(hdr, sizeof(int), 5, fp) != 5 || hdr[1] != num_ranks) {
        fclose(fp);
        if (chdir(cwd)) {}
        return -1;
    }
    int *start = (int *)calloc((size_t)num_ranks + 1, sizeof(int));
    if (fread(start, sizeof(int), (size_t)num_ranks, fp) != (size_t)num_ranks) {
        fclose(fp);
        free(start);
        if (chdir(cwd)) {}
        return -1;
    }
    fclose(fp);
    start[num_ranks] = hdr[0];
    shim_set_world(num_ranks);
    ref_job *jobs = (ref_job *)calloc((size_t)num_ranks, sizeof(ref_job));
    pthread_t *th = (pthread_t *)calloc((size_t)num_ranks, sizeof(pthread_t));
    for (int r = 0; r < num_ranks; r++) {
        jobs[r].rank = r;
        jobs[r].it_max = it_max;
        jobs[r].save = save;
        jobs[r].save_every = save_every;
        jobs[r].tau = tau;
        jobs[r].set_tau = (tau == tau);
        jobs[r].force = force;
        jobs[r].set_force = (force == force);
        jobs[r].start = start;
        jobs[r].f0 = f0;
        jobs[r].f1 = f1;
        jobs[r].mac = mac;
        jobs[r].num_f = hdr[0];
        pthread_create(&th[r], NULL, ref_rank_main, &jobs[r]);
    }
    double el = 0.0;
    for (int r = 0; r < num_ranks; r++) {
        pthread_join(th[r], NULL);
        if (jobs[r].elapsed > el) el = jobs[r].elapsed;
    }
    if (elapsed) *elapsed = el;
    free(jobs);
    free(th);
    free(start);
    shim_set_world(1);
    if (chdir(cwd)) {}
    return 0;
}
