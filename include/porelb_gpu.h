/*
 * porelb_gpu.h - C ABI of the GB300 sparse-lattice D3Q19 BGK solver.
 *
 * This is the drop-in boundary for porelb's hot path.  The reference has no
 * plugin or FFI layer: its "interface" is the SIMULATION* function set of one
 * C executable (porelb.h:127-165), the V.bin node table written by preprocess
 * (preprocess.c:166-193) and the part_%03d_%07d.bin macro dumps
 * (porelb.c:375-391).  Each entry point below names the reference function or
 * file format it replaces.
 *
 * Conventions
 *   - Every call returns an int status (PLB_OK == 0, negative on error); no
 *     call exits the process.  The negative codes keep the reference's exit
 *     codes where one exists (-6 density guard, porelb.c:338-342).
 *   - Host buffers are caller-owned.  Device memory is owned by the handle.
 *   - One CUDA stream per handle; a handle is not thread-safe.
 *   - Nothing here takes a torch type; plain pointers and sizes only.
 */
#ifndef PORELB_GPU_H_
#define PORELB_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PLB_Q 19

/* Neighbour entry, byte-compatible with NEIGHBOR_INFO (porelb.h:58-62):
 * type@0, padding@1, pid@2, id@4; 8 bytes. */
typedef struct {
    uint8_t node_type;
    uint8_t pad_;
    uint16_t node_pid;
    uint32_t node_id;
} plb_neighbor_info;

/* Fluid-node record, byte-compatible with NODE_INFO (porelb.h:73-76):
 * x@0 y@2 z@4, padding@6, nb_info[18]@8; 152 bytes.  nb_info[i] describes
 * the node at (x,y,z)+e[i+1], periodic (preprocess.c:133-151). */
typedef struct {
    uint16_t x, y, z;
    uint16_t pad_;
    plb_neighbor_info nb_info[PLB_Q - 1];
} plb_node_info;

/* enum NEIGHBOR_TYPE (porelb.h:55) */
enum { PLB_TYPE_FLUID = 0, PLB_TYPE_SOLID = 1, PLB_TYPE_EXTERN = 2 };

/* Status codes. */
enum {
    PLB_OK = 0,
    PLB_ERR_ARG = -1,      /* bad argument / size */
    PLB_ERR_IO = -2,       /* file open/read/write (porelb.c:18-22,65-69) */
    PLB_ERR_TABLE = -3,    /* node table fails the check_V bounds test (porelb.c:115-141) */
    PLB_ERR_CUDA = -4,     /* CUDA runtime error or no device */
    PLB_ERR_NOMEM = -5,    /* host or device allocation failed */
    PLB_ERR_DENSITY = -6,  /* density guard rho>1.2 | rho<0.5 (porelb.c:338-342) */
    PLB_ERR_NUMP = -7,     /* num_p inconsistent with the table (porelb.c:29-34) */
    PLB_ERR_STATE = -8     /* call out of order (e.g. step before init) */
};

/* Storage / arithmetic form of the distributions. */
enum {
    PLB_FP64_EXACT = 0, /* FP64 storage, reference operation order, no FMA: bit-exact */
    PLB_FP64 = 1,       /* FP64 storage, collision in exact Q60 fixed point on
                           the integer pipes (within 1e-12 of the reference) */
    PLB_FP32 = 2,       /* FP32 storage, FP32 collision */
    PLB_FP16DEV = 3,    /* scaled FP16 deviations f_i - w_i, FP32 collision */
    PLB_BF16DEV = 4,    /* scaled BF16 deviations f_i - w_i, FP32 collision */
    PLB_FP64_FMA = 5    /* FP64 storage, FMA-contracted FP64 collision */
};

/* Node ordering in device memory (the same results in every order).
 * REFERENCE is the table's own row order (x fastest, then y, then z): a
 * warp's 32 consecutive nodes then have their neighbours in every direction
 * in one shifted run of nodes, which gathers best while the three z-planes
 * a step reads at once stay in L2.  MORTON keeps the gathers local at any
 * size.  AUTO takes REFERENCE when three z-planes of the domain's nodes
 * (their distributions, words and numbering) fit in 60% of the L2, else
 * MORTON
 * (256^3: row order, FP64 17.2 against 16.4 GLUPS; 512^3 FP16 and FP32: row
 * order; 512^3 and 1024^3 FP64: Morton). */
enum { PLB_ORDER_MORTON = 0, PLB_ORDER_REFERENCE = 1, PLB_ORDER_AUTO = 2 };
/* The order AUTO picks for n nodes in an nx*ny*nz domain with elem-byte
 * storage on device `device`. */
int plb_auto_ordering(long long n, int nz, int elem_bytes, int device);

/* Wall rule. */
enum {
    PLB_BOUNDARY_REFERENCE = 0, /* porelb's link bounce-back as written
                                   (porelb.c:296-297): the bounced value lands
                                   in f1[x][j] instead of f1[x][re j], so some
                                   slots are written twice and others never */
    PLB_BOUNDARY_HALFWAY = 1    /* standard half-way bounce-back: a population
                                   that would stream into a solid cell returns
                                   to its node reversed; conserves mass */
};

/* Halo semantics for tables written with num_p > 1. */
enum {
    PLB_HALO_AUTO = -1,        /* REMOTE_WINS when num_p > 1, else SINGLE */
    PLB_HALO_SINGLE = 0,       /* one-rank run: last writer in node order wins */
    PLB_HALO_REMOTE_WINS = 1   /* mpirun -np num_p: a cross-slab push overwrites
                                  the local bounce-back write (porelb.c:430-433) */
};

typedef struct {
    double tau;      /* relaxation time; reference hard-codes 0.8 (porelb.c:87) */
    double force_x;  /* body force along x; reference hard-codes 1e-3 (porelb.c:91) */
    int precision;   /* PLB_FP64_EXACT ... */
    int ordering;    /* PLB_ORDER_AUTO (default), PLB_ORDER_MORTON or
                        PLB_ORDER_REFERENCE */
    int halo;        /* PLB_HALO_* */
    int block_size;  /* threads per block for the step kernel; 0 = default */
    int device;      /* CUDA device ordinal */
    int boundary;    /* PLB_BOUNDARY_REFERENCE (default) or PLB_BOUNDARY_HALFWAY */
    int kernel_variant; /* register budget of the step kernel: 0 (or 2) =
                           default (PLB_FP64: 128 registers, 16 warps per SM;
                           FP32/16-bit forms: 48 registers); 1 = 80 registers
                           (PLB_FP64) or unconstrained; 3 = 64 (PLB_FP64) or 40
                           registers.  Ignored by the other FP64 forms. */
    int l2_prefetch; /* L2 prefetch of the nodes of the blocks half a wave
                        of resident blocks ahead:
                        0 = the form's default (on for PLB_FP64, where it
                        pays; off for the bandwidth-bound forms), 1 = on,
                        -1 = off */
    int reserved[4];
} plb_params;

typedef struct plb_sim plb_sim;

/* ---------------------------------------------------------------- tables */

/* Fill *p with the reference defaults: tau 0.8, force 1e-3 (init_para,
 * porelb.c:83-94), FP64_EXACT, automatic node order and halo semantics. */
void plb_default_params(plb_params *p);

/* Replaces build_V (preprocess.c:29-164).  flag is nx*ny*nz uint8, x fastest,
 * 1 = fluid, 0 = solid.  With out == NULL only *num_node is computed.
 * v_sub_start receives num_p ints.  Requires nz % num_p == 0 (the reference
 * writes out of bounds otherwise, preprocess.c:107).  Fields that the
 * reference leaves defined are reproduced bit-exactly; SOLID entries carry the
 * previous node's id/pid the way the reference's reused temporary does and
 * padding bytes are zero. */
int plb_build_table(const uint8_t *flag, int nx, int ny, int nz, int num_p,
                    plb_node_info *out, int *num_node, int *v_sub_start);

/* Replaces save_V (preprocess.c:166-193): header int32 num_node, num_p, nx,
 * ny, nz; int32 v_sub_start[num_p]; NODE_INFO[num_node]. */
int plb_write_vbin(const char *path, const plb_node_info *V, int num_node,
                   int num_p, int nx, int ny, int nz, const int *v_sub_start);

/* Replaces the V.bin reader of alloc_memory (porelb.c:15-81), for all ranks
 * at once.  Read the header first, allocate, then read the body. */
int plb_read_vbin_header(const char *path, int *num_node, int *num_p, int *nx,
                         int *ny, int *nz);
int plb_read_vbin(const char *path, plb_node_info *V, int *v_sub_start);

/* Replaces check_V (porelb.c:115-141) with strict bounds (x < nx rather than
 * the reference's x > nx test) and id checks on FLUID/EXTERN entries. */
int plb_check_table(const plb_node_info *V, int num_node, int nx, int ny,
                    int nz, int num_p, const int *v_sub_start);

/* Deterministic periodic sphere pack (the geometry source of the benchmark
 * configurations; the reference reads flag.bin from outside).  splitmix64
 * stream from `seed`; each sphere draws centre x, y, z uniform in [0,n) and
 * radius rmin + (rmax-rmin)*u; a cell (x,y,z) is solid iff its periodic
 * minimum-image squared distance to a centre is <= R*R.  Spheres are added
 * until the fluid fraction is <= porosity.  flag receives nx*ny*nz bytes. */
int plb_sphere_pack(uint64_t seed, int nx, int ny, int nz, double rmin,
                    double rmax, double porosity, uint8_t *flag,
                    int *num_spheres, double *porosity_out);

/* ---------------------------------------------------------------- solver */

/* alloc_memory + check_V + init_para + build_send_recv_info
 * (porelb.c:15-222): uploads the table, builds the pull table and the node
 * permutation on the device, allocates the distributions.  V is num_node
 * records in V.bin order (rank slabs concatenated in pid order). */
int plb_create(const plb_node_info *V, int num_node, int nx, int ny, int nz,
               int num_p, const int *v_sub_start, const plb_params *p,
               plb_sim **out);
void plb_destroy(plb_sim *sim);

/* build_V + plb_create in one device pass, from a flag grid (host buffer,
 * values 0/1, x fastest; num_p z slabs as preprocess.c:107).  No V.bin
 * records are formed: fluid cells are ranked in lexicographic order (the
 * reference node numbers) and along the Morton curve on the device.  The
 * handle is identical to plb_create on plb_build_table's output. */
int plb_create_from_flag(const uint8_t *flag, int nx, int ny, int nz,
                         int num_p, const plb_params *p, plb_sim **out);

/* plb_sphere_pack on the device: the same flag bit for bit (flag may be
 * NULL to only report the sphere count and porosity). */
int plb_sphere_pack_device(uint64_t seed, int nx, int ny, int nz, double rmin,
                           double rmax, double porosity, int device,
                           uint8_t *flag, int *num_spheres, double *porosity_out);

/* Sphere pack + table build + handle, all on the device. */
int plb_create_packed(uint64_t seed, int nx, int ny, int nz, double rmin,
                      double rmax, double porosity, int num_p,
                      const plb_params *p, plb_sim **out, int *num_spheres,
                      double *porosity_out);

/* init_dist_macro (porelb.c:224-238): rho=1, u=0, f0=f1=feq. */
int plb_init_equilibrium(plb_sim *sim);

/* nsteps iterations of the loop body of main (porelb.c:426-437): stream,
 * halo (on-device), collide, with the half-force shift for it > 0
 * (porelb.c:347-348).  Iterations are it_begin .. it_begin+nsteps-1.
 * plb_step waits for the device and reports the density guard; the _async
 * form only enqueues, and plb_sync waits and reports. */
int plb_step(plb_sim *sim, int it_begin, int nsteps);
int plb_step_async(plb_sim *sim, int it_begin, int nsteps);
int plb_sync(plb_sim *sim);

/* Rho, Ux, Uy, Uz of the last step, in reference node order (save_data,
 * porelb.c:375-391).  Any pointer may be NULL. */
int plb_get_macros(plb_sim *sim, double *rho, double *ux, double *uy,
                   double *uz);

/* save_data (porelb.c:375-391): writes part_%03d_%07d.bin for every rank of
 * the table into dir (NULL = current directory), tagged `tag`. */
int plb_save_parts(plb_sim *sim, const char *dir, int tag);

/* Post-collision distributions f0 as reference AoS f[i*19+j], reference
 * node order, converted to FP64 for the reduced-precision forms. */
int plb_get_f(plb_sim *sim, double *f_aos);
/* Overwrite the state from a reference-order AoS array. */
int plb_set_f(plb_sim *sim, const double *f_aos);
/* The distributions the next step will collide, after its stream: the
 * reference's f1 after the next stream_inner_nodes (porelb.c:285-300) of
 * the current f0, AoS, reference node order, FP64. */
int plb_get_f_streamed(plb_sim *sim, double *f_aos);

/* FP64 sums over the last step's macros: sum of Ux and of Rho. */
int plb_reduce(plb_sim *sim, double *sum_ux, double *mass);

/* Permeability k = <u_x> * nu / F.  k_darcy uses the superficial mean
 * sum(Ux)/(nx*ny*nz); k_intrinsic uses sum(Ux)/num_node.  nu =(tau-1/2)/3
 * (porelb.c:89).  Either pointer may be NULL. */
int plb_permeability(plb_sim *sim, double *k_darcy, double *k_intrinsic);

/* Details of the last density-guard trip: the iteration, node index in
 * reference order, its coordinates and rho.  Returns PLB_OK if none. */
int plb_last_error(plb_sim *sim, int *it, int *node, int *x, int *y, int *z,
                   double *rho);

/* What the step kernel reported since plb_init_equilibrium, read at each
 * synchronising call: PLB_FLAG_FX_FALLBACK when a node's populations left
 * the range of the form's fast arithmetic and the node was recomputed with
 * native FP64 operations (the fixed-point form: populations far from the
 * weights; the bit-exact form: values or a density outside [2^-64, 2^64),
 * exact zeros included).  Results keep the form's accuracy either way.  No
 * reference counterpart (the reference has one form). */
#define PLB_FLAG_FX_FALLBACK 2u
int plb_kernel_flags(plb_sim *sim, unsigned *flags);

/* Sizes and the handle's CUDA stream (a cudaStream_t). */
int plb_info(plb_sim *sim, int *num_node, int *npad, int *precision,
             size_t *device_bytes);
void *plb_stream(plb_sim *sim);

/* ---------------------------------------------------------------- batch */

/* Many independent samples in one device node pool (no reference
 * counterpart; each sample runs porelb's step loop).  Samples are admitted
 * into free 256-node block ranges, stepped together K steps at a time (one
 * CUDA graph per interval), checked for steady state after each interval
 * (|<u_x>(t) - <u_x>(t-K)| <= tol |<u_x>(t)|) and retired. */
typedef struct plb_batch plb_batch;

typedef struct {
    double tau;          /* relaxation time of the sample */
    double force_x;      /* body force of the sample */
    double tol;          /* steady-state tolerance on <u_x> over one interval */
    long long max_steps; /* stop after this many steps (<= 0: no limit) */
    double handoff_tol;  /* > tol: park the sample (status 4, blocks kept)
                            once its change is below this, for
                            plb_batch_transfer; 0 = never */
    int reserved[2];
} plb_sample_params;

/* Device bytes per pool node for a storage form (the admission unit). */
size_t plb_batch_bytes_per_node(int precision, int keep_macros);
/* capacity_nodes: pool size; check_every: interval K (even); keep_macros: also
 * keep rho/u per node for plb_batch_get_macros. */
int plb_batch_create(size_t capacity_nodes, int max_samples, int precision,
                     int check_every, int keep_macros, int device,
                     plb_batch **out);
/* Pool parameters with the launch choices the tuner makes (zero = the
 * library default for each choice). */
typedef struct {
    size_t capacity_nodes; /* pool size */
    int max_samples;
    int precision;         /* PLB_FP64 ... */
    int check_every;       /* interval K (even) */
    int keep_macros;
    int device;
    int cta_threads;       /* batch-step CTA: 128 or 256 threads (0: 128 for
                              PLB_FP64, 256 otherwise) */
    int l2_prefetch;       /* L2 prefetch of the pool block half a wave
                              ahead: 0 = default (on for PLB_FP64), 1 on,
                              -1 off */
    int ordering;          /* node order within each sample:
                              PLB_ORDER_MORTON (0, default),
                              PLB_ORDER_REFERENCE or PLB_ORDER_AUTO (chosen
                              per sample) */
    int l2_group_kb;       /* L2 groups: samples whose working set (both
                              distribution buffers and the neighbour words)
                              fits this many KiB are packed into groups, and
                              an interval runs its K steps one group at a
                              time while the group stays in L2; larger
                              samples step together first.  0 = off (the
                              default), -1 = 60% of the device's L2.  Results
                              are the same bits either way. */
    int reserved[4];
} plb_batch_params;
int plb_batch_create_ex(const plb_batch_params *p, plb_batch **out);
void plb_batch_destroy(plb_batch *b);
/* Admit a sample from a host flag grid (0/1) or a device sphere pack.
 * PLB_ERR_NOMEM when no free range or sample slot is left. */
int plb_batch_add_flag(plb_batch *b, const uint8_t *flag, int nx, int ny,
                       int nz, const plb_sample_params *sp, int *id);
int plb_batch_add_packed(plb_batch *b, uint64_t seed, int nx, int ny, int nz,
                         double rmin, double rmax, double porosity,
                         const plb_sample_params *sp, int *id,
                         int *num_spheres, double *porosity_out);
/* Run `intervals` intervals of K steps (stops early when nothing is active):
 * plb_batch_launch + plb_batch_finish each. */
int plb_batch_run(plb_batch *b, int intervals, int *n_active);
/* Start one interval on the pool's stream and return (*n_active: samples it
 * steps; 0 = nothing launched).  While it runs the caller may admit samples
 * (built on a second stream; they join at the next launch), poll, read
 * results and transfer parked samples; plb_batch_get_f / get_macros and
 * releasing a sample the interval steps return PLB_ERR_STATE. */
int plb_batch_launch(plb_batch *b, int *n_active);
/* Wait for the interval in flight, then check every sample it stepped:
 * converged, step limit, density guard or handoff tolerance. */
int plb_batch_finish(plb_batch *b);
/* Admit into dst a sample parked in src (same device and K; deviation
 * storage forms): its node table and current state, converted to dst's
 * storage form, with its step count and convergence history, which the
 * steady-state test continues from.  The caller then releases it in src.
 * No reference counterpart. */
int plb_batch_transfer(plb_batch *src, int id, plb_batch *dst, int *new_id);
/* Device time of the last completed interval (CUDA events around its graph
 * on the pool's stream), in milliseconds. */
int plb_batch_interval_ms(plb_batch *b, float *ms);
/* Ids of samples that finished since the last poll. */
int plb_batch_poll(plb_batch *b, int *ids, int max_ids, int *count);
/* status: 0 running, 1 converged, 2 step limit, 3 released, 4 parked at the
 * handoff tolerance, <0 error. */
int plb_batch_result(plb_batch *b, int id, double *k_darcy, double *mean_ux,
                     long long *steps, int *status);
int plb_batch_release(plb_batch *b, int id);
int plb_batch_get_f(plb_batch *b, int id, double *f_aos);
int plb_batch_get_macros(plb_batch *b, int id, double *rho, double *ux,
                         double *uy, double *uz);
int plb_batch_info(plb_batch *b, long long *t, int *active,
                   long long *used_nodes, long long *capacity_nodes,
                   size_t *device_bytes);
int plb_batch_sample_nodes(plb_batch *b, int id, int *num_node);
/* Room left in the pool, in nodes: the largest free block range (0 when no
 * sample slot is free) and all free ranges together.  A sample of n fluid
 * nodes can be admitted now when ceil(n / 256) * 256 <= *largest_range. */
int plb_batch_free_nodes(plb_batch *b, long long *largest_range,
                         long long *total);
void *plb_batch_stream(plb_batch *b);

/* ------------------------------------------------------- no allocation */

/* No counterpart in the reference.  Sum of ux[0..n) and of rho[0..n)
 * (caller's device arrays) into out[0], out[1] (caller's device memory), on
 * `stream` (a cudaStream_t, NULL = legacy default), without allocating: for
 * callers that cannot let a library allocate device memory (a framework
 * that owns all device memory through its own pool and budget, a serving
 * loop admitting work against a fixed HBM budget, code that must not
 * synchronise the device the way cudaMalloc/cudaFree can).  Its per-block
 * partial sums live in one fixed 4 MiB device array that every GPU loading
 * this library holds until exit, so n is limited to
 * PLB_REDUCE_NOALLOC_MAX_NODES (larger n: PLB_ERR_ARG, nothing launched).
 * Calls share that array: calls that overlap on the GPU race.  The first
 * call on a device looks up the array's device address; make it before any
 * stream capture.  That address is kept for the life of the process: it
 * assumes the device's primary context is not reset while the library is
 * in use (after cudaDeviceReset, or a primary-context reset through the
 * driver API, the module may load at another address and later calls would
 * use a stale one).  Asynchronous: out is valid once the stream reaches it. */
#define PLB_REDUCE_NOALLOC_MAX_NODES 67108864LL
int plb_reduce_noalloc(const double *ux, const double *rho, long long n,
                       double *out, void *stream);

/* ------------------------------------------------------ fault injection */

/* Test hooks, no reference counterpart (the reference exits on a failed
 * allocation, porelb.c:18-22,65-69).  Every device allocation the library
 * makes is counted; after plb_fault_inject_alloc(n) with n > 0 the n-th
 * allocation from then on fails once with PLB_ERR_NOMEM semantics (no
 * cudaMalloc is called, so the GPU is not touched); n <= 0 disarms it.
 * plb_alloc_count returns the allocations made so far, so that a test can
 * count a call's allocations and fail each one in turn. */
int plb_fault_inject_alloc(long long nth);
long long plb_alloc_count(void);

/* Human-readable text for a status code. */
const char *plb_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif /* PORELB_GPU_H_ */
