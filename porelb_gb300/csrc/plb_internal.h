/*
 * plb_internal.h - shared definitions of the CUDA translation units.
 */
#ifndef PLB_INTERNAL_H_
#define PLB_INTERNAL_H_

#include <cuda_runtime.h>
#include <stdint.h>

#include "porelb_gpu.h"
#include "plb_fx.h"

/* Every device allocation of the library goes through here, so that a test
 * can make one of them fail on the host (plb_fault_inject_alloc) and drive
 * the out-of-memory paths without touching the GPU. */
cudaError_t plb_dev_malloc(void **p, size_t bytes);
template <typename P>
static inline cudaError_t plb_cuda_malloc(P **p, size_t bytes)
{
    return plb_dev_malloc((void **)p, bytes);
}

namespace plb {

constexpr int Q = 19;

/* D3Q19 set in the reference order (porelb.h:10-50) as constexpr functions:
 * inside fully unrolled loops they fold to immediates. */
__host__ __device__ constexpr int ex(int j)
{
    return (j == 1 || j == 12 || j == 14 || j == 16 || j == 18) ? 1
         : (j == 2 || j == 11 || j == 13 || j == 15 || j == 17) ? -1 : 0;
}
__host__ __device__ constexpr int ey(int j)
{
    return (j == 3 || j == 7 || j == 10 || j == 15 || j == 18) ? 1
         : (j == 4 || j == 8 || j == 9 || j == 16 || j == 17) ? -1 : 0;
}
__host__ __device__ constexpr int ez(int j)
{
    return (j == 5 || j == 7 || j == 9 || j == 12 || j == 13) ? 1
         : (j == 6 || j == 8 || j == 10 || j == 11 || j == 14) ? -1 : 0;
}
/* re[] (porelb.h:44-50): 1<->2, 3<->4, ... */
__host__ __device__ constexpr int opp(int j)
{
    return j == 0 ? 0 : ((j & 1) ? j + 1 : j - 1);
}
/* weight class: 0 -> 1/3, 1 -> 1/18, 2 -> 1/36 */
__host__ __device__ constexpr int wclass(int j)
{
    return j == 0 ? 0 : (j <= 6 ? 1 : 2);
}

/* A neighbour word is the signed 32-bit offset, counted from the start of
 * plane j of the distribution array, of the value node i pulls for
 * direction j: the source node s (0 <= s < npad) of the pull, or for a
 * bounce-back node i's own value of direction re(j) = j +- 1, which lies at
 * i + (re(j) - j) * npad.  One address computation serves both.  Node index
 * N (the "rest slot") holds the initial value of every direction and is
 * never written: links no push or bounce ever writes read it.  Offsets need
 * 2 * npad < 2^31, hence kMaxNodes. */
constexpr long long kMaxNodes = (1LL << 30) - 512;

__host__ __device__ inline uint32_t bounce_word(int j, long long i, long long npad)
{
    return (uint32_t)(i + (long long)(opp(j) - j) * npad);
}

/* Per-solve collision coefficients (host-computed from tau and F). */
struct Coeffs {
    /* FP64, in the reference's operation order */
    double omega, om1, k3, force, half_force;
    /* FP32 forms (rounded from the FP64 values) */
    float omega_f, om1_f, c_f, half_force_f;
    float scale, inv_scale; /* deviation storage scale */
    fx::Consts fxk;         /* fixed-point form */
    int it;                 /* iteration number (the it > 0 rule) */
    /* bit-exact form: a run constant outside the range of the integer
     * multiply's node check (every node then takes the native multiply) */
    int exact_native;
};

struct StepArgs {
    const void *fin;
    void *fout;
    const uint32_t *nbr;  /* [18][npad] */
    const int *perm;      /* new -> reference index (density guard report) */
    long long npad;
    int n;
    Coeffs co;
    /* macros (rho, ux, uy, uz; stride npad) and per-block sums, or NULL */
    double *macro;
    double *partial;  /* [2][gridDim.x]: sum ux, sum rho */
    unsigned long long *err; /* min over (it << 32 | reference index) */
    unsigned int *flags;     /* bit 0: FP16 scale overflow, bit 1: fallback */
    int pf_blocks;           /* L2 prefetch distance in blocks (0 = none) */
};

/* One sample of a batch (device copy). */
struct SampleDev {
    Coeffs co;
    long long base; /* first node of the sample in the pool */
    int n;          /* fluid nodes */
    int start;      /* batch step at which the sample started */
};

struct BatchArgs {
    const void *fin;
    void *fout;
    const uint32_t *nbr;
    long long npad;
    const int *blk_list;       /* pool blocks this launch covers (one CTA each,
                                  two for 128-thread CTAs) */
    const int *blk_sample;     /* per 256-node pool block: sample << 9 | nodes of
                                  the sample in the block, -1 = free */
    long long part_stride;     /* pool blocks: stride of the partial-sum rows */
    const SampleDev *samples;
    const int *t_base;         /* batch step counter (device) */
    int t_off;                 /* this launch's step = *t_base + t_off */
    double *macro;             /* may be NULL */
    double *partial;           /* [3][part_stride] by pool block: sum ux, sum rho,
                                  max |stored deviation| */
    unsigned int *serr;        /* per-sample error bits */
    int pf_blocks;             /* L2 prefetch distance in CTAs (0 = none) */
    /* L2 groups: when grp is set, the launch steps group *grp_cur only,
     * pool blocks blk_list[grp[2g] .. grp[2g] + grp[2g + 1]) */
    const int *grp;
    const int *grp_cur;
};

/* Exclusive scan of m uint32 counts into offs (device memory). */
int scan_words(const uint32_t *cnt, uint32_t *offs, size_t m, cudaStream_t st);

/* Device geometry (plb_geom.cu). */
int sphere_pack_device(uint64_t seed, int nx, int ny, int nz, double rmin,
                       double rmax, double porosity, uint8_t *dflag,
                       int *num_spheres, double *porosity_out, cudaStream_t st);
int flag_rank(const uint8_t *dflag, int nx, int ny, int nz, int num_p,
              uint32_t *lexbits, uint32_t *lexoffs, int *n, int *slab_start,
              cudaStream_t st);
int flag_tables(const uint8_t *dflag, int nx, int ny, int nz, int num_p,
                int ordering, int remote_wins, int halfway, const uint32_t *lexbits,
                const uint32_t *lexoffs, int n, long long npad, int *perm,
                uint16_t *coord, uint32_t *nbr, uint32_t word_base,
                uint32_t rest_word, cudaStream_t st);

/* Launch one step of the given precision. */
/* blocks of the step kernel resident on the device at once (0 if unknown) */
int step_wave_blocks(int precision, int block, int variant);
/* the same for the batch step kernel with CTAs of `cta` threads */
int batch_wave_blocks(int precision, int cta);
/* default threads per CTA of the batch step (128 or 256) */
int batch_default_cta(int precision);
cudaError_t launch_step(int precision, bool macros, const StepArgs &a,
                        int block, int variant, cudaStream_t s);

/* The batch step kernel (one BatchArgs argument) of a storage form with
 * CTAs of `cta` threads (128 or 256; pool blocks of 256 nodes, 256 / cta
 * CTAs each), for a graph kernel node; NULL for another size. */
constexpr int kBatchBlock = 256;
const void *batch_step_kernel(int precision, bool macros, int cta);

/* Fill the coefficients from tau, F and the storage scale. */
void make_coeffs(double tau, double force, float scale, Coeffs *c);

}  // namespace plb

#endif
