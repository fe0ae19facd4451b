/*
 * mpi.h - in-process MPI shim used only to compile the reference porelb
 * sources into the test oracle (oracle/_ref).  Ranks are threads of one
 * process; point-to-point messages are buffered copies matched FIFO per
 * (source, destination, tag).  It implements exactly the calls the reference
 * makes (porelb.c:405-441): Init, Finalize, Comm_rank, Comm_size, Wtime,
 * Sendrecv, Isend, Irecv, Waitall.  TEST INFRASTRUCTURE ONLY.
 */
#ifndef ORACLE_MPI_SHIM_H_
#define ORACLE_MPI_SHIM_H_

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef struct {
    int MPI_SOURCE;
    int MPI_TAG;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

#ifdef __cplusplus
extern "C" {
#endif
int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm c, int *rank);
int MPI_Comm_size(MPI_Comm c, int *size);
double MPI_Wtime(void);
int MPI_Sendrecv(const void *sbuf, int scount, MPI_Datatype st, int dest,
                 int stag, void *rbuf, int rcount, MPI_Datatype rt, int src,
                 int rtag, MPI_Comm c, MPI_Status *status);
int MPI_Isend(const void *buf, int count, MPI_Datatype t, int dest, int tag,
              MPI_Comm c, MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype t, int src, int tag,
              MPI_Comm c, MPI_Request *req);
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *statuses);

/* shim control: world size and the calling thread's rank */
void shim_set_world(int size);
void shim_set_rank(int rank);
#ifdef __cplusplus
}
#endif
#endif
