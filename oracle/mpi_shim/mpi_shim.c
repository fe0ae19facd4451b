/*
 * mpi_shim.c - threads-as-ranks implementation of the MPI subset the
 * reference uses.  TEST INFRASTRUCTURE ONLY.
 */
#include "mpi.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct msg {
    int src, dst, tag;
    size_t bytes;
    void *data;
    struct msg *next;
} msg;

typedef struct {
    int used;
    void *buf;
    size_t bytes;
    int src, tag;
} pending_recv;

#define MAX_PENDING 4096

static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t g_cv = PTHREAD_COND_INITIALIZER;
static msg *g_head = NULL, *g_tail = NULL;
static int g_size = 1;
static __thread int t_rank = 0;
static __thread pending_recv t_pending[MAX_PENDING];

void shim_set_world(int size) { g_size = size; }
void shim_set_rank(int rank) { t_rank = rank; }

static size_t type_size(MPI_Datatype t) { return t == MPI_DOUBLE ? 8 : 4; }

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm c, int *rank) { (void)c; *rank = t_rank; return 0; }
int MPI_Comm_size(MPI_Comm c, int *size) { (void)c; *size = g_size; return 0; }

double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int MPI_Isend(const void *buf, int count, MPI_Datatype t, int dest, int tag,
              MPI_Comm c, MPI_Request *req)
{
    (void)c;
    msg *m = (msg *)calloc(1, sizeof(msg));
    m->src = t_rank;
    m->dst = dest;
    m->tag = tag;
    m->bytes = (size_t)count * type_size(t);
    m->data = malloc(m->bytes ? m->bytes : 1);
    memcpy(m->data, buf, m->bytes);
    pthread_mutex_lock(&g_mu);
    if (g_tail) g_tail->next = m;
    else g_head = m;
    g_tail = m;
    pthread_cond_broadcast(&g_cv);
    pthread_mutex_unlock(&g_mu);
    if (req) *req = -1; /* buffered: complete */
    return 0;
}

int MPI_Irecv(void *buf, int count, MPI_Datatype t, int src, int tag,
              MPI_Comm c, MPI_Request *req)
{
    (void)c;
    for (int k = 0; k < MAX_PENDING; k++)
        if (!t_pending[k].used) {
            t_pending[k].used = 1;
            t_pending[k].buf = buf;
            t_pending[k].bytes = (size_t)count * type_size(t);
            t_pending[k].src = src;
            t_pending[k].tag = tag;
            *req = k;
            return 0;
        }
    abort();
}

static void complete_recv(int k)
{
    pending_recv *p = &t_pending[k];
    pthread_mutex_lock(&g_mu);
    for (;;) {
        msg *prev = NULL;
        for (msg *m = g_head; m; prev = m, m = m->next) {
            if (m->dst == t_rank && m->src == p->src && m->tag == p->tag) {
                if (prev) prev->next = m->next;
                else g_head = m->next;
                if (g_tail == m) g_tail = prev;
                pthread_mutex_unlock(&g_mu);
                memcpy(p->buf, m->data, m->bytes < p->bytes ? m->bytes : p->bytes);
                free(m->data);
                free(m);
                p->used = 0;
                return;
            }
        }
        pthread_cond_wait(&g_cv, &g_mu);
    }
}

int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *statuses)
{
    (void)statuses;
    for (int i = 0; i < n; i++)
        if (reqs[i] >= 0) {
            complete_recv(reqs[i]);
            reqs[i] = -1;
        }
    return 0;
}

int MPI_Sendrecv(const void *sbuf, int scount, MPI_Datatype st, int dest,
                 int stag, void *rbuf, int rcount, MPI_Datatype rt, int src,
                 int rtag, MPI_Comm c, MPI_Status *status)
{
    (void)status;
    MPI_Request r;
    MPI_Isend(sbuf, scount, st, dest, stag, c, NULL);
    MPI_Irecv(rbuf, rcount, rt, src, rtag, c, &r);
    MPI_Waitall(1, &r, NULL);
    return 0;
}
