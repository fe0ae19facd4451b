/*
 * porelb_oracle.h - CPU restatement of porelb's sparse-lattice D3Q19 BGK path.
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the checker for the GPU library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  The product path never calls it.
 *
 * Parity pin: every function here is checked bit-exactly against the
 * reference itself, compiled from its own sources by oracle/Makefile into
 * oracle/_ref/ (tests/test_oracle.py), and the committed golden
 * fixtures in tests/golden/ were written by that compiled reference.
 */
#ifndef PORELB_ORACLE_H_
#define PORELB_ORACLE_H_

#include <stdint.h>
#include "../include/porelb_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* build_V restated (preprocess.c:29-164).  See the C file for details. */
int orc_build_v(const uint8_t *flag, int nx, int ny, int nz, int num_p,
                plb_node_info *out, int *num_node, int *v_sub_start);

typedef struct orc_sim orc_sim;

/* Create a solver over the whole table (all rank slabs).  num_p ranks are
 * emulated with the reference's z-slab semantics; threads > 1 runs the ranks
 * (or, for num_p == 1, nothing extra) on that many host threads. */
orc_sim *orc_create(const plb_node_info *V, int num_node, int nx, int ny,
                    int nz, int num_p, const int *v_sub_start, double tau,
                    double force_x);
void orc_destroy(orc_sim *s);
void orc_init(orc_sim *s);                       /* porelb.c:224-238 */
/* Run steps it_begin..it_begin+nsteps-1 with the push-form stream and the
 * collision.  Returns 0, or -6 with *bad_node / *bad_it set when the density
 * guard trips (porelb.c:338-342).  threads <= 1 runs serially. */
int orc_run(orc_sim *s, int it_begin, int nsteps, int threads, int *bad_it,
            int *bad_node);
/* One stream phase only (porelb.c:285-300 plus the remote-push unpack of
 * porelb.c:302-312), for f1 checks. */
void orc_stream(orc_sim *s);
int orc_collide(orc_sim *s, int it, int *bad_node); /* porelb.c:318-365 */
double *orc_f0(orc_sim *s);
double *orc_f1(orc_sim *s);
double *orc_macro(orc_sim *s, int which); /* 0 rho, 1 ux, 2 uy, 3 uz */
int orc_num_node(orc_sim *s);

/* Pull-form restatement: for each node i and direction j=1..18, where f1[i][j]
 * comes from after one push stream.  kind[i*18+j-1]: 0 = f0[src][j],
 * 1 = f0[i][re j], 2 = never written (keeps its previous f1 value).  src is a
 * global node index. */
void orc_pull_table(const plb_node_info *V, int num_node, int num_p,
                    const int *v_sub_start, int remote_wins, uint8_t *kind,
                    uint32_t *src);
/* As orc_pull_table; halfway != 0 gives the standard half-way bounce-back
 * (every slot written once: pull from s if fluid, else f0[i][re j]). */
void orc_pull_table_rule(const plb_node_info *V, int num_node, int num_p,
                         const int *v_sub_start, int remote_wins, int halfway,
                         uint8_t *kind, uint32_t *src);

/* One fused pull-stream + collide step on AoS arrays using that table:
 * f1 := stream(f0) (kind 2 slots untouched), then collide f1 -> f0. */
int orc_pull_step(const uint8_t *kind, const uint32_t *src, int num_node,
                  double *f0, double *f1, double *rho, double *ux, double *uy,
                  double *uz, double tau, double force_x, int it,
                  int *bad_node);

/* The synthetic sphere-pack generator (splitmix64, periodic minimum image,
 * spheres added until the porosity reaches the target): flag is nx*ny*nz
 * bytes, x fastest, 1 fluid / 0 solid.  The same field as the library's
 * plb_sphere_pack, written independently. */
int orc_sphere_pack(uint64_t seed, int nx, int ny, int nz, double rmin,
                    double rmax, double porosity, uint8_t *flag,
                    int *num_spheres, double *porosity_out);

/* Sum of Ux and Rho in node order (FP64, serial). */
void orc_reduce(orc_sim *s, double *sum_ux, double *mass);

#ifdef __cplusplus
}
#endif
#endif
