/*
 * porelb_oracle.c - CPU restatement of porelb's sparse-lattice D3Q19 BGK path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library, never the thing
 * measured or shipped.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it (as liborc.so, built by oracle/Makefile).
 *
 * It restates, in the reference's own operation order, the functions of the
 * hot path:
 *   build_V            preprocess.c:29-164
 *   init_dist_macro    porelb.c:224-238
 *   stream_inner_nodes porelb.c:285-300
 *   update_recv_dist   porelb.c:302-312 (halo unpack after the local stream)
 *   collision + feq    porelb.c:318-365, porelb.c:6-13
 * Compile with -ffp-contract=off: the reference is built as ISO C99, which
 * disables FMA contraction, and its results are reproduced bit for bit.
 *
 * Ranks of an mpirun run are emulated in one address space: the table is the
 * concatenation of all rank slabs (V.bin order) and a push across a slab
 * boundary is applied after every rank's local stream, as the reference's
 * MPI_Waitall + update_recv_dist order makes it (porelb.c:428-433).
 *
 * Parity pin: tests/test_oracle.py compares this file with the
 * reference compiled from its own sources (oracle/_ref/), byte for byte.
 */
#include "porelb_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define Q 19

/* D3Q19 velocities, weights and opposite directions in the reference's order
 * (porelb.h:10-50). */
static const int E[Q][3] = {
    {0, 0, 0},   {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
    {0, 0, 1},   {0, 0, -1},  {0, 1, 1},  {0, -1, -1}, {0, -1, 1},
    {0, 1, -1},  {-1, 0, -1}, {1, 0, 1},  {-1, 0, 1}, {1, 0, -1},
    {-1, 1, 0},  {1, -1, 0},  {-1, -1, 0}, {1, 1, 0}};
static const double W[Q] = {
    1.0 / 3,  1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18,
    1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
    1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};
static const int OPP[Q] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9,
                           12, 11, 14, 13, 16, 15, 18, 17};

/* ------------------------------------------------------------------ build_V */

/* build_V (preprocess.c:29-164).  Fluid nodes are numbered in (z,y,x)
 * lexicographic order (preprocess.c:74-82,99-113); rank pid = z/(nz/num_p)
 * (preprocess.c:107); each node's record lands at v_sub_start[pid] +
 * position-within-rank (preprocess.c:154).  nb_info[i] describes the node at
 * x+e[i+1] with periodic wrap (preprocess.c:133-151): a zero flag makes it
 * SOLID and leaves id/pid as they were for the previous node (the reference
 * reuses one temporary record); any other flag value makes it FLUID (same
 * rank) or EXTERN with its position-within-rank and rank. */
int orc_build_v(const uint8_t *flag, int nx, int ny, int nz, int num_p,
                plb_node_info *out, int *num_node, int *v_sub_start)
{
    if (!flag || nx <= 0 || ny <= 0 || nz <= 0 || num_p <= 0 || num_p > nz ||
        nz % num_p != 0 || !num_node)
        return PLB_ERR_ARG;
    const long size = (long)nx * ny * nz;
    int *x_to_n = (int *)calloc((size_t)size, sizeof(int));
    if (!x_to_n) return PLB_ERR_NOMEM;
    int n = 0;
    for (long k = 0; k < size; k++)
        if (flag[k] == 1) x_to_n[k] = n++;
    *num_node = n;
    if (!out) {
        free(x_to_n);
        return PLB_OK;
    }
    int *node_pid = (int *)malloc(sizeof(int) * (size_t)(n ? n : 1));
    int *node_pos = (int *)malloc(sizeof(int) * (size_t)(n ? n : 1));
    int *count = (int *)calloc((size_t)num_p, sizeof(int));
    if (!node_pid || !node_pos || !count) {
        free(x_to_n); free(node_pid); free(node_pos); free(count);
        return PLB_ERR_NOMEM;
    }
    const int slab = nz / num_p;
    int i = 0;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                long k = ((long)z * ny + y) * nx + x;
                if (flag[k] != 1) continue;
                node_pid[i] = z / slab;
                node_pos[i] = count[node_pid[i]]++;
                i++;
            }
    if (v_sub_start) {
        v_sub_start[0] = 0;
        for (int p = 1; p < num_p; p++)
            v_sub_start[p] = v_sub_start[p - 1] + count[p - 1];
    }
    int *start = (int *)calloc((size_t)num_p, sizeof(int));
    for (int p = 1; p < num_p; p++) start[p] = start[p - 1] + count[p - 1];

    plb_node_info rec;
    memset(&rec, 0, sizeof(rec));
    i = 0;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                long k = ((long)z * ny + y) * nx + x;
                if (flag[k] != 1) continue;
                rec.x = (uint16_t)x;
                rec.y = (uint16_t)y;
                rec.z = (uint16_t)z;
                const int p = node_pid[i];
                for (int d = 0; d < Q - 1; d++) {
                    int xp = (x + E[d + 1][0] + nx) % nx;
                    int yp = (y + E[d + 1][1] + ny) % ny;
                    int zp = (z + E[d + 1][2] + nz) % nz;
                    long kp = ((long)zp * ny + yp) * nx + xp;
                    if (flag[kp] == 0) {
                        rec.nb_info[d].node_type = PLB_TYPE_SOLID;
                    } else {
                        int g = x_to_n[kp];
                        int pp = node_pid[g];
                        rec.nb_info[d].node_id = (uint32_t)node_pos[g];
                        rec.nb_info[d].node_pid = (uint16_t)pp;
                        rec.nb_info[d].node_type =
                            (uint8_t)(pp == p ? PLB_TYPE_FLUID : PLB_TYPE_EXTERN);
                    }
                }
                out[start[p] + node_pos[i]] = rec;
                i++;
            }
    free(start);
    free(count);
    free(node_pos);
    free(node_pid);
    free(x_to_n);
    return PLB_OK;
}

/* ------------------------------------------------------------------- solver */

struct orc_sim {
    int N, nx, ny, nz, num_p;
    const plb_node_info *V;
    int *start;   /* v_sub_start[num_p + 1] */
    int *rank_of; /* rank of each global node */
    double tau, omega, force;
    double *f0, *f1, *rho, *ux, *uy, *uz;
    /* cross-slab links: f1[dst*Q+j] = f0[src*Q+j] after the local stream */
    int nlink;
    int *link_src, *link_dst, *link_j;
};

/* feq (porelb.c:6-13), same operation order. */
static inline double feq(int k, double rho, double u, double v, double w)
{
    double eu = E[k][0] * u + E[k][1] * v + E[k][2] * w;
    double uv = u * u + v * v + w * w;
    return W[k] * rho * (1.0 + 3 * eu + 4.5 * eu * eu - 1.5 * uv);
}

orc_sim *orc_create(const plb_node_info *V, int num_node, int nx, int ny,
                    int nz, int num_p, const int *v_sub_start, double tau,
                    double force_x)
{
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    if (!s) return NULL;
    s->N = num_node;
    s->nx = nx; s->ny = ny; s->nz = nz;
    s->num_p = num_p;
    s->V = V;
    s->tau = tau;
    s->omega = 1.0 / tau;   /* porelb.c:88 */
    s->force = force_x;
    s->start = (int *)calloc((size_t)num_p + 1, sizeof(int));
    for (int p = 0; p < num_p; p++) s->start[p] = v_sub_start ? v_sub_start[p] : 0;
    s->start[num_p] = num_node;
    size_t nq = (size_t)num_node * Q;
    s->f0 = (double *)calloc(nq ? nq : 1, sizeof(double));
    s->f1 = (double *)calloc(nq ? nq : 1, sizeof(double));
    s->rho = (double *)calloc(num_node ? num_node : 1, sizeof(double));
    s->ux = (double *)calloc(num_node ? num_node : 1, sizeof(double));
    s->uy = (double *)calloc(num_node ? num_node : 1, sizeof(double));
    s->uz = (double *)calloc(num_node ? num_node : 1, sizeof(double));
    s->rank_of = (int *)calloc(num_node ? num_node : 1, sizeof(int));
    for (int p = 0; p < num_p; p++)
        for (int i = s->start[p]; i < s->start[p + 1]; i++) s->rank_of[i] = p;
    int nl = 0;
    for (int i = 0; i < num_node; i++)
        for (int d = 0; d < Q - 1; d++)
            if (V[i].nb_info[d].node_type == PLB_TYPE_EXTERN) nl++;
    s->nlink = nl;
    s->link_src = (int *)calloc(nl ? nl : 1, sizeof(int));
    s->link_dst = (int *)calloc(nl ? nl : 1, sizeof(int));
    s->link_j = (int *)calloc(nl ? nl : 1, sizeof(int));
    nl = 0;
    for (int i = 0; i < num_node; i++)
        for (int d = 0; d < Q - 1; d++)
            if (V[i].nb_info[d].node_type == PLB_TYPE_EXTERN) {
                s->link_src[nl] = i;
                s->link_dst[nl] = s->start[V[i].nb_info[d].node_pid] +
                                  (int)V[i].nb_info[d].node_id;
                s->link_j[nl] = d + 1;
                nl++;
            }
    return s;
}

void orc_destroy(orc_sim *s)
{
    if (!s) return;
    free(s->start); free(s->rank_of);
    free(s->f0); free(s->f1);
    free(s->rho); free(s->ux); free(s->uy); free(s->uz);
    free(s->link_src); free(s->link_dst); free(s->link_j);
    free(s);
}

/* init_dist_macro (porelb.c:224-238). */
void orc_init(orc_sim *s)
{
    for (int i = 0; i < s->N; i++) {
        s->rho[i] = 1.0;
        s->ux[i] = 0.0;
        s->uy[i] = 0.0;
        s->uz[i] = 0.0;
        for (int j = 0; j < Q; j++)
            s->f0[(size_t)i * Q + j] = s->f1[(size_t)i * Q + j] =
                feq(j, s->rho[i], s->ux[i], s->uy[i], s->uz[i]);
    }
}

/* stream_inner_nodes over nodes [lo, hi) of one rank (porelb.c:285-300).
 * FLUID ids are positions within the same rank. */
static void stream_range(orc_sim *s, int lo, int hi)
{
    const double *f0 = s->f0;
    double *f1 = s->f1;
    for (int i = lo; i < hi; i++) {
        const int base = s->start[s->rank_of[i]];
        f1[(size_t)i * Q] = f0[(size_t)i * Q];
        for (int j = 1; j < Q; j++) {
            const plb_neighbor_info nb = s->V[i].nb_info[j - 1];
            if (nb.node_type == PLB_TYPE_FLUID)
                f1[((size_t)base + nb.node_id) * Q + j] = f0[(size_t)i * Q + j];
            else if (nb.node_type == PLB_TYPE_SOLID)
                f1[(size_t)i * Q + j] = f0[(size_t)i * Q + OPP[j]];
        }
    }
}

static void unpack_range(orc_sim *s, int lo, int hi)
{
    for (int l = lo; l < hi; l++)
        s->f1[(size_t)s->link_dst[l] * Q + s->link_j[l]] =
            s->f0[(size_t)s->link_src[l] * Q + s->link_j[l]];
}

void orc_stream(orc_sim *s)
{
    stream_range(s, 0, s->N);
    unpack_range(s, 0, s->nlink);
}

/* collision (porelb.c:318-365) over nodes [lo, hi); returns the first node
 * failing the density guard, or -1. */
static int collide_range(orc_sim *s, int it, int lo, int hi)
{
    const double omega = s->omega;
    const double F = s->force;
    for (int i = lo; i < hi; i++) {
        const double *g = s->f1 + (size_t)i * Q;
        double rho = 0.0, rhou = 0.0, rhov = 0.0, rhow = 0.0;
        for (int j = 0; j < Q; j++) {
            rho += g[j];
            rhou += E[j][0] * g[j];
            rhov += E[j][1] * g[j];
            rhow += E[j][2] * g[j];
        }
        if (rho > 1.2 || rho < 0.5) return i;
        if (it > 0) rhou += 0.5 * F;
        double u = rhou / rho, v = rhov / rho, w = rhow / rho;
        s->rho[i] = rho;
        s->ux[i] = u;
        s->uy[i] = v;
        s->uz[i] = w;
        double *h = s->f0 + (size_t)i * Q;
        for (int j = 0; j < Q; j++)
            h[j] = (1.0 - omega) * g[j] +
                   (omega + (1.0 - 0.5 * omega) * 3.0 * (E[j][0] - u) * F) *
                       feq(j, rho, u, v, w);
    }
    return -1;
}

int orc_collide(orc_sim *s, int it, int *bad_node)
{
    int b = collide_range(s, it, 0, s->N);
    if (bad_node) *bad_node = b;
    return b >= 0 ? PLB_ERR_DENSITY : PLB_OK;
}

/* Threaded run: thread t owns ranks [t*P/T, (t+1)*P/T) and the cross-slab
 * links whose source it owns.  Phases per step: local stream | unpack |
 * collide, separated by barriers, which is the order of main's loop body
 * (porelb.c:428-434). */
typedef struct {
    orc_sim *s;
    int t, T, it_begin, nsteps;
    int node_lo, node_hi, link_lo, link_hi;
    pthread_barrier_t *bar;
    volatile int *stop;
    int *bad_it, *bad_node;
    pthread_mutex_t *mu;
} orc_worker;

static void *orc_worker_main(void *arg)
{
    orc_worker *w = (orc_worker *)arg;
    for (int k = 0; k < w->nsteps; k++) {
        const int it = w->it_begin + k;
        stream_range(w->s, w->node_lo, w->node_hi);
        pthread_barrier_wait(w->bar);
        unpack_range(w->s, w->link_lo, w->link_hi);
        pthread_barrier_wait(w->bar);
        int b = collide_range(w->s, it, w->node_lo, w->node_hi);
        if (b >= 0) {
            pthread_mutex_lock(w->mu);
            if (*w->bad_it < 0 || it < *w->bad_it ||
                (it == *w->bad_it && b < *w->bad_node)) {
                *w->bad_it = it;
                *w->bad_node = b;
            }
            *w->stop = 1;
            pthread_mutex_unlock(w->mu);
        }
        pthread_barrier_wait(w->bar);
        if (*w->stop) break;
    }
    return NULL;
}

int orc_run(orc_sim *s, int it_begin, int nsteps, int threads, int *bad_it,
            int *bad_node)
{
    int bi = -1, bn = -1;
    if (threads <= 1 || s->num_p <= 1) {
        for (int k = 0; k < nsteps; k++) {
            orc_stream(s);
            int b = collide_range(s, it_begin + k, 0, s->N);
            if (b >= 0) { bi = it_begin + k; bn = b; break; }
        }
    } else {
        int T = threads < s->num_p ? threads : s->num_p;
        pthread_t *th = (pthread_t *)calloc((size_t)T, sizeof(pthread_t));
        orc_worker *w = (orc_worker *)calloc((size_t)T, sizeof(orc_worker));
        pthread_barrier_t bar;
        pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
        volatile int stop = 0;
        pthread_barrier_init(&bar, NULL, (unsigned)T);
        int l = 0;
        for (int t = 0; t < T; t++) {
            int p_lo = (int)((long)t * s->num_p / T);
            int p_hi = (int)((long)(t + 1) * s->num_p / T);
            w[t].s = s; w[t].t = t; w[t].T = T;
            w[t].it_begin = it_begin; w[t].nsteps = nsteps;
            w[t].node_lo = s->start[p_lo];
            w[t].node_hi = s->start[p_hi];
            w[t].link_lo = l;
            while (l < s->nlink && s->link_src[l] < w[t].node_hi) l++;
            w[t].link_hi = l;
            w[t].bar = &bar; w[t].stop = &stop; w[t].mu = &mu;
            w[t].bad_it = &bi; w[t].bad_node = &bn;
        }
        for (int t = 0; t < T; t++)
            pthread_create(&th[t], NULL, orc_worker_main, &w[t]);
        for (int t = 0; t < T; t++) pthread_join(th[t], NULL);
        pthread_barrier_destroy(&bar);
        free(th);
        free(w);
    }
    if (bad_it) *bad_it = bi;
    if (bad_node) *bad_node = bn;
    return bn >= 0 ? PLB_ERR_DENSITY : PLB_OK;
}

double *orc_f0(orc_sim *s) { return s->f0; }
double *orc_f1(orc_sim *s) { return s->f1; }
double *orc_macro(orc_sim *s, int which)
{
    switch (which) {
    case 0: return s->rho;
    case 1: return s->ux;
    case 2: return s->uy;
    default: return s->uz;
    }
}
int orc_num_node(orc_sim *s) { return s->N; }

void orc_reduce(orc_sim *s, double *sum_ux, double *mass)
{
    double a = 0.0, m = 0.0;
    for (int i = 0; i < s->N; i++) {
        a += s->ux[i];
        m += s->rho[i];
    }
    if (sum_ux) *sum_ux = a;
    if (mass) *mass = m;
}

/* ---------------------------------------------------------------- pull form */

/* Where f1[i][j] comes from after one push stream (porelb.c:285-312).
 * The slot is written by the push of s = x - e_j when s is fluid, and by the
 * bounce-back of x itself when t = x + e_j is solid.  nb_info[re(j)-1]
 * describes s, nb_info[j-1] describes t.  When both write, the later one in
 * node order wins (push iff s comes after x); with remote_wins a push across
 * slabs wins always, since update_recv_dist runs after the local stream. */
void orc_pull_table(const plb_node_info *V, int num_node, int num_p,
                    const int *v_sub_start, int remote_wins, uint8_t *kind,
                    uint32_t *src)
{
    orc_pull_table_rule(V, num_node, num_p, v_sub_start, remote_wins, 0, kind, src);
}

/* halfway != 0: the standard half-way bounce-back instead of the
 * reference's rule: pull from s when s is fluid, else the node's own
 * reversed population. */
void orc_pull_table_rule(const plb_node_info *V, int num_node, int num_p,
                         const int *v_sub_start, int remote_wins, int halfway,
                         uint8_t *kind, uint32_t *src)
{
    int *start = (int *)calloc((size_t)num_p + 1, sizeof(int));
    for (int p = 0; p < num_p; p++) start[p] = v_sub_start ? v_sub_start[p] : 0;
    start[num_p] = num_node;
    int rank = 0;
    for (int i = 0; i < num_node; i++) {
        while (rank + 1 < num_p && i >= start[rank + 1]) rank++;
        for (int j = 1; j < Q; j++) {
            const plb_neighbor_info sn = V[i].nb_info[OPP[j] - 1];
            const plb_neighbor_info tn = V[i].nb_info[j - 1];
            const int push = sn.node_type != PLB_TYPE_SOLID;
            const int bounce = tn.node_type == PLB_TYPE_SOLID;
            long sg = -1;
            if (sn.node_type == PLB_TYPE_FLUID) sg = (long)start[rank] + sn.node_id;
            else if (sn.node_type == PLB_TYPE_EXTERN)
                sg = (long)start[sn.node_pid] + sn.node_id;
            uint8_t k;
            if (halfway) k = push ? 0 : 1;
            else if (push && !bounce) k = 0;
            else if (!push && bounce) k = 1;
            else if (!push && !bounce) k = 2;
            else if (remote_wins && sn.node_type == PLB_TYPE_EXTERN) k = 0;
            else k = (sg > i) ? 0 : 1;
            kind[(size_t)i * 18 + j - 1] = k;
            src[(size_t)i * 18 + j - 1] = (uint32_t)(k == 0 ? sg : i);
        }
    }
    free(start);
}

int orc_pull_step(const uint8_t *kind, const uint32_t *src, int num_node,
                  double *f0, double *f1, double *rho, double *ux, double *uy,
                  double *uz, double tau, double force_x, int it, int *bad_node)
{
    for (int i = 0; i < num_node; i++) {
        f1[(size_t)i * Q] = f0[(size_t)i * Q];
        for (int j = 1; j < Q; j++) {
            const uint8_t k = kind[(size_t)i * 18 + j - 1];
            if (k == 0)
                f1[(size_t)i * Q + j] = f0[(size_t)src[(size_t)i * 18 + j - 1] * Q + j];
            else if (k == 1)
                f1[(size_t)i * Q + j] = f0[(size_t)i * Q + OPP[j]];
        }
    }
    orc_sim tmp;
    memset(&tmp, 0, sizeof(tmp));
    tmp.N = num_node;
    tmp.omega = 1.0 / tau;
    tmp.force = force_x;
    tmp.f0 = f0; tmp.f1 = f1;
    tmp.rho = rho; tmp.ux = ux; tmp.uy = uy; tmp.uz = uz;
    int b = collide_range(&tmp, it, 0, num_node);
    if (bad_node) *bad_node = b;
    return b >= 0 ? PLB_ERR_DENSITY : PLB_OK;
}

/* -------------------------------------------------------------- geometry */

/* The synthetic geometry generator, restated from its definition (the
 * reference reads flag.bin from outside and has no generator of its own):
 * a splitmix64 stream (Steele, Lea & Flood, OOPSLA 2014) seeded with the
 * configuration seed; each sphere draws its centre uniform in [0,n) per
 * axis (x, y, z) and then its radius uniform in [rmin, rmax], each uniform
 * from the top 53 bits of one draw; a cell is solid iff its periodic
 * minimum-image squared distance to the centre, summed x then y then z, is
 * at most r^2; spheres are added while the fluid fraction is above the
 * target porosity.  Written independently of the library's generator so
 * that the CPU baseline builds its input without the library; a CPU test
 * checks the two give the same flag field byte for byte. */
static uint64_t orc_mix(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double orc_unit(uint64_t *s)
{
    return (double)(orc_mix(s) >> 11) / 9007199254740992.0; /* 2^53 */
}

/* the distinct cells of [c - r, c + r] on a periodic axis of n cells, each
 * with its minimum-image distance to c; returns the count */
static int orc_axis_cells(double c, double r, int n, int *cell, double *dist)
{
    long lo = (long)floor(c - r), hi = (long)ceil(c + r);
    if (hi - lo + 1 > n) hi = lo + n - 1;
    int m = 0;
    for (long k = lo; k <= hi; k++) {
        const int idx = (int)(((k % n) + n) % n);
        double d = fabs((double)idx - c);
        if ((double)n - d < d) d = (double)n - d;
        cell[m] = idx;
        dist[m] = d;
        m++;
    }
    return m;
}

int orc_sphere_pack(uint64_t seed, int nx, int ny, int nz, double rmin,
                    double rmax, double porosity, uint8_t *flag,
                    int *num_spheres, double *porosity_out)
{
    if (!flag || nx <= 0 || ny <= 0 || nz <= 0 || !(rmin > 0.0) ||
        rmax < rmin || !(porosity >= 0.0) || !(porosity <= 1.0))
        return PLB_ERR_ARG;
    const size_t cells = (size_t)nx * ny * nz;
    for (size_t k = 0; k < cells; k++) flag[k] = 1;
    int nmax = nx > ny ? nx : ny;
    if (nz > nmax) nmax = nz;
    int *cx = malloc(sizeof(int) * (size_t)nmax * 3);
    double *dx = malloc(sizeof(double) * (size_t)nmax * 3);
    if (!cx || !dx) {
        free(cx);
        free(dx);
        return PLB_ERR_NOMEM;
    }
    int *cy = cx + nmax, *cz = cx + 2 * nmax;
    double *dy = dx + nmax, *dz = dx + 2 * nmax;
    uint64_t st = seed;
    size_t solid = 0;
    int count = 0;
    while ((double)(cells - solid) / (double)cells > porosity && count < 100000000) {
        const double px = orc_unit(&st) * nx;
        const double py = orc_unit(&st) * ny;
        const double pz = orc_unit(&st) * nz;
        const double r = rmin + (rmax - rmin) * orc_unit(&st);
        count++;
        const int mx = orc_axis_cells(px, r, nx, cx, dx);
        const int my = orc_axis_cells(py, r, ny, cy, dy);
        const int mz = orc_axis_cells(pz, r, nz, cz, dz);
        for (int c = 0; c < mz; c++)
            for (int b = 0; b < my; b++) {
                uint8_t *row = flag + ((size_t)cz[c] * ny + cy[b]) * nx;
                for (int a = 0; a < mx; a++) {
                    const double d2 = dx[a] * dx[a] + dy[b] * dy[b] + dz[c] * dz[c];
                    if (!(d2 <= r * r) || !row[cx[a]]) continue;
                    row[cx[a]] = 0;
                    solid++;
                }
            }
    }
    free(cx);
    free(dx);
    if (num_spheres) *num_spheres = count;
    if (porosity_out) *porosity_out = (double)(cells - solid) / (double)cells;
    return PLB_OK;
}
