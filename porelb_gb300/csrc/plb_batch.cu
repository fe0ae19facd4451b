/*
 * plb_batch.cu - many independent porous samples in one device pool.
 *
 * Samples of uneven size are concatenated as 256-node block ranges of one
 * node pool; a per-block map names the sample whose tau, force and storage
 * scale the step applies (k_batch_step, plb_step.cu).  All samples advance
 * together: one launch per lattice step covers every active block, and an
 * interval of K steps (the last writing the per-block sums) plus the
 * per-sample reduction are CUDA graphs, built once and replayed;
 * admissions and retirements only change the active-block list and the
 * grid of the step nodes.  On request (l2_group_kb) the samples that fit
 * a budget are packed into L2 groups, and the interval steps each group
 * K times while it stays in L2, replaying one group chain per group.  An
 * interval is launched asynchronously (plb_batch_launch) and completed by
 * plb_batch_finish, which checks each
 * sample's steady-state criterion (relative change of the mean u_x over
 * the interval), retires converged samples and frees their blocks.
 * Samples admitted while an interval runs are built on a second stream into
 * free block ranges (first fit) and join at the next launch.  A sample may
 * instead be parked at a looser handoff tolerance, keeping its blocks, and
 * moved into another pool (plb_batch_transfer), e.g. from 16-bit to FP32
 * storage.  A sample's arithmetic does not depend on what else is in the
 * pool, so its result is the same alone and in a mix.
 *
 * The reference has no batching; each sample follows its own step loop
 * (porelb.c:426-437) with the it > 0 half-force rule counted from the
 * sample's admission.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <map>
#include <type_traits>
#include <vector>

#include "plb_internal.h"

using namespace plb;

namespace {

constexpr int B = kBatchBlock;

size_t elem_of(int precision)
{
    switch (precision) {
    case PLB_FP64_EXACT:
    case PLB_FP64:
    case PLB_FP64_FMA: return 8;
    case PLB_FP32: return 4;
    case PLB_FP16DEV:
    case PLB_BF16DEV: return 2;
    default: return 0;
    }
}

__device__ __forceinline__ double wq(int j)
{
    return j == 0 ? 1.0 / 3 : (j <= 6 ? 1.0 / 18 : 1.0 / 36);
}

/* rest state over [lo, hi) of both buffers: w_j (FP64 forms) or 0 */
__global__ void k_fill_rest(void *f0, void *f1, long long npad, long long lo,
                            long long hi, int elem)
{
    const long long k = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= hi) return;
    for (int j = 0; j < Q; j++) {
        const long long o = j * npad + k;
        if (elem == 8) {
            ((double *)f0)[o] = wq(j);
            ((double *)f1)[o] = wq(j);
        } else if (elem == 4) {
            ((float *)f0)[o] = 0.f;
            ((float *)f1)[o] = 0.f;
        } else {
            ((uint16_t *)f0)[o] = 0;
            ((uint16_t *)f1)[o] = 0;
        }
    }
}

/* block map of pool blocks [lo, lo + cnt): sample sid (<< 9) and the
 * number of its `nodes` that fall in each block; sid < 0 frees them */
__global__ void k_set_blocks(int *blk, long long lo, long long cnt, int sid, long long nodes)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cnt) return;
    const long long in = nodes - k * B;
    blk[lo + k] = sid < 0 ? -1 : (sid << 9) | (int)(in < B ? (in > 0 ? in : 0) : B);
}

__global__ void k_advance(int *t, int by) { *t += by; }

/* per-sample sums of the per-block partials, in block order (one CTA per
 * sample slot): ssum[s] = {sum ux, sum rho, max |stored deviation|} */
__global__ void k_sample_sums(const SampleDev *sp, const int *active,
                              const double *partial, int nb, int h, double *ssum)
{
    const int s = blockIdx.x;
    __shared__ double su[32], sr[32], sd[32];
    double tu = 0.0, tr = 0.0, td = 0.0;
    if (active[s]) {
        /* h partial rows per pool block, nb rows in all */
        const long long b0 = sp[s].base / B * h;
        const long long b1 = (sp[s].base + sp[s].n + B - 1) / B * h;
        for (long long b = b0 + threadIdx.x; b < b1 && b < nb; b += blockDim.x) {
            tu += partial[b];
            tr += partial[nb + b];
            td = fmax(td, partial[2 * nb + b]);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        tu += __shfl_down_sync(0xffffffffu, tu, o);
        tr += __shfl_down_sync(0xffffffffu, tr, o);
        td = fmax(td, __shfl_down_sync(0xffffffffu, td, o));
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { su[wid] = tu; sr[wid] = tr; sd[wid] = td; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, r = 0.0, d = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            a += su[k];
            r += sr[k];
            d = fmax(d, sd[k]);
        }
        ssum[3 * s] = a;
        ssum[3 * s + 1] = r;
        ssum[3 * s + 2] = d;
    }
}

/* multiply the stored deviations of [lo, hi) by factor (16-bit forms) */
template <typename T>
__global__ void k_rescale(T *f, long long npad, long long lo, long long hi, float factor)
{
    const long long k = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= hi) return;
    for (int j = 0; j < Q; j++) {
        T *p = f + j * npad + k;
        if constexpr (sizeof(T) == 2 && std::is_same<T, __half>::value)
            *p = __float2half_rn(__half2float(*p) * factor);
        else
            *p = __float2bfloat16_rn(__bfloat162float(*p) * factor);
    }
}

template <typename T>
__device__ __forceinline__ double ld_dev(const T *p);
template <> __device__ __forceinline__ double ld_dev<float>(const float *p) { return *p; }
template <> __device__ __forceinline__ double ld_dev<__half>(const __half *p) { return __half2float(*p); }
template <> __device__ __forceinline__ double ld_dev<__nv_bfloat16>(const __nv_bfloat16 *p) { return __bfloat162float(*p); }

/* f of one sample, reference order, AoS FP64 */
template <typename T>
__global__ void k_get_f_sample(const T *f, long long npad, long long base, int n,
                               const int *perm, float inv_scale, double *out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long i = base + k;
    const long long o = (long long)perm[i] * Q;
    for (int j = 0; j < Q; j++) {
        if constexpr (sizeof(T) == 8) {
            out[o + j] = ((const double *)f)[j * npad + i];
        } else {
            const double g = ld_dev<T>(f + j * npad + i) * (double)inv_scale;
            out[o + j] = wq(j) + wq(j) * g;
        }
    }
}

__global__ void k_get_macro_sample(const double *macro, long long npad, long long base,
                                   int n, const int *perm, double *out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long i = base + k;
    const long long o = perm[i];
    for (int c = 0; c < 4; c++) out[c * (long long)n + o] = macro[c * npad + i];
}

/* a sample's node table moved into another pool: pull words re-based */
__global__ void k_translate_words(const uint32_t *src, long long snp, long long sbase,
                                  uint32_t srest, uint32_t *dst, long long dnp,
                                  long long dbase, uint32_t drest, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    for (int j = 1; j < Q; j++) {
        const uint32_t w = src[(long long)(j - 1) * snp + sbase + k];
        uint32_t o;
        if (w == srest) o = drest;
        else if ((long long)(uint32_t)(w - (uint32_t)sbase) < (long long)n)
            o = (uint32_t)(dbase + (long long)(w - (uint32_t)sbase));
        else o = bounce_word(j, dbase + k, dnp);
        dst[(long long)(j - 1) * dnp + dbase + k] = o;
    }
}

/* a sample's stored deviations moved into another storage form: g =
 * stored / scale_in, stored again as g * scale_out */
template <typename TI, typename TO>
__global__ void k_convert_dev(const TI *in, long long inp, long long ibase, float inv_in,
                              TO *out, long long onp, long long obase, float scale_out,
                              int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    for (int j = 0; j < Q; j++) {
        const float g = (float)ld_dev<TI>(in + j * inp + ibase + k) * inv_in;
        const float h = g * scale_out;
        TO *p = out + j * onp + obase + k;
        if constexpr (std::is_same<TO, float>::value) *p = h;
        else if constexpr (std::is_same<TO, __half>::value) *p = __float2half_rn(h);
        else *p = __float2bfloat16_rn(h);
    }
}

struct SampleHost {
    int used = 0, active = 0, finished = 0;
    int parked = 0;    /* stopped at the handoff tolerance, blocks kept */
    int stepping = 0;  /* stepped by the interval in flight */
    int pending = 0;   /* admitted; joins at the next launch */
    long long blk0 = 0, nblk = 0;
    int n = 0, nx = 0, ny = 0, nz = 0;
    double tau = 0, force = 0, tol = 0, nu = 0, handoff_tol = 0;
    long long max_steps = 0;
    long long start = 0, steps = 0;
    int checks = 0;
    double ux = 0, prev_ux = 0, mass = 0, k_darcy = 0;
    float scale = 1.f;
    int status = 0;
    SampleDev dev;
};

unsigned gb(long long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

struct plb_batch {
    int device = 0, precision = 0, K = 1000, keep_macros = 0, max_samples = 0;
    size_t elem = 0;
    cudaStream_t st = nullptr;
    cudaStream_t adm = nullptr; /* admissions, concurrent with an interval */
    cudaEvent_t ev0 = nullptr, ev1 = nullptr; /* around the interval in flight */
    float last_ms = 0.f;
    bool in_flight = false;
    int cta = 256;     /* threads per CTA of the batch step */
    int ordering = PLB_ORDER_MORTON; /* node order of each sample's table */
    int prefetch = 0;  /* L2 prefetch of the pool block half a wave ahead */
    long long cap_blocks = 0, npad = 0, rest = 0;
    void *f[2] = {nullptr, nullptr};
    int cur = 0;
    uint32_t *nbr = nullptr;
    int *perm = nullptr;
    uint16_t *coord = nullptr;
    double *macro = nullptr;
    int *blk = nullptr;
    SampleDev *sdev = nullptr;
    int *sactive = nullptr;
    double *partial = nullptr;
    double *ssum = nullptr;
    unsigned *serr = nullptr;
    int *t_dev = nullptr;
    double *h_ssum = nullptr;   /* pinned */
    unsigned *h_serr = nullptr; /* pinned */
    long long t = 0;
    int *blist = nullptr;          /* device: active pool blocks */
    std::vector<int> hlist;        /* host copy */
    bool list_dirty = true;
    std::map<long long, long long> free_blocks; /* start -> length */
    std::vector<SampleHost> s;
    std::vector<int> done;
    /* K steps over the blocks of the samples outside the L2 groups */
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int graph_cur = -1;
    int graph_grid = 0;                     /* grid of the step nodes */
    std::vector<BatchArgs> step_args;       /* kernel arguments per step node */
    std::vector<cudaGraphNode_t> step_nodes;
    /* L2 groups: samples whose working set fits group_bytes are packed into
     * groups, and the interval steps one group K times while it stays in
     * L2, then the next (0 = no groups) */
    size_t group_bytes = 0;
    std::vector<int> hgroups;               /* {first list entry, blocks} */
    int *dgroups = nullptr;                 /* device copy */
    int *gcur = nullptr;                    /* device: the group being stepped */
    int big_blocks = 0, group_blocks_max = 0;
    cudaGraph_t graph_grp = nullptr;        /* K steps of group *gcur, then ++*gcur */
    cudaGraphExec_t gexec_grp = nullptr;
    int grp_grid = 0;
    std::vector<BatchArgs> grp_args;
    std::vector<cudaGraphNode_t> grp_nodes;
    cudaGraphExec_t gexec_tail = nullptr;   /* step counter, sums, read-back */
    size_t bytes = 0;
};

#define BCK(call)                                                           \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                            \
            fprintf(stderr, "porelb_gpu: %s failed: %s\n", #call,           \
                    cudaGetErrorString(e_));                                \
            return e_ == cudaErrorMemoryAllocation ? PLB_ERR_NOMEM : PLB_ERR_CUDA; \
        }                                                                   \
    } while (0)

size_t plb_batch_bytes_per_node(int precision, int keep_macros)
{
    const size_t e = elem_of(precision);
    if (!e) return 0;
    /* 2 x 19 distributions, 18 words, perm, 3 coordinates, macros */
    return 2 * Q * e + 72 + 4 + 6 + (keep_macros ? 32 : 0);
}

static void batch_free(plb_batch *b)
{
    if (!b) return;
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->gexec_grp) cudaGraphExecDestroy(b->gexec_grp);
    if (b->graph_grp) cudaGraphDestroy(b->graph_grp);
    if (b->gexec_tail) cudaGraphExecDestroy(b->gexec_tail);
    cudaFree(b->dgroups);
    cudaFree(b->gcur);
    cudaFree(b->f[0]);
    cudaFree(b->f[1]);
    cudaFree(b->nbr);
    cudaFree(b->perm);
    cudaFree(b->coord);
    cudaFree(b->macro);
    cudaFree(b->blk);
    cudaFree(b->blist);
    cudaFree(b->sdev);
    cudaFree(b->sactive);
    cudaFree(b->partial);
    cudaFree(b->ssum);
    cudaFree(b->serr);
    cudaFree(b->t_dev);
    if (b->h_ssum) cudaFreeHost(b->h_ssum);
    if (b->h_serr) cudaFreeHost(b->h_serr);
    if (b->st) cudaStreamDestroy(b->st);
    if (b->adm) cudaStreamDestroy(b->adm);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    delete b;
}

void plb_batch_destroy(plb_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->adm) cudaStreamSynchronize(b->adm);
    batch_free(b);
}

int plb_batch_create(size_t capacity_nodes, int max_samples, int precision,
                     int check_every, int keep_macros, int device,
                     plb_batch **out)
{
    plb_batch_params bp;
    memset(&bp, 0, sizeof(bp));
    bp.capacity_nodes = capacity_nodes;
    bp.max_samples = max_samples;
    bp.precision = precision;
    bp.check_every = check_every;
    bp.keep_macros = keep_macros;
    bp.device = device;
    return plb_batch_create_ex(&bp, out);
}

int plb_batch_create_ex(const plb_batch_params *bp, plb_batch **out)
{
    if (!out || !bp) return PLB_ERR_ARG;
    *out = nullptr;
    const size_t capacity_nodes = bp->capacity_nodes;
    const int max_samples = bp->max_samples, precision = bp->precision;
    const int check_every = bp->check_every, keep_macros = bp->keep_macros;
    const int device = bp->device;
    if ((bp->cta_threads != 0 && bp->cta_threads != 128 && bp->cta_threads != B) ||
        bp->l2_prefetch < -1 || bp->l2_prefetch > 1 || bp->l2_group_kb < -1 ||
        (bp->ordering != PLB_ORDER_MORTON && bp->ordering != PLB_ORDER_REFERENCE &&
         bp->ordering != PLB_ORDER_AUTO))
        return PLB_ERR_ARG;
    if (capacity_nodes == 0 || max_samples <= 0 || max_samples > (1 << 22) ||
        elem_of(precision) == 0 ||
        check_every <= 0 || (check_every & 1) || capacity_nodes >= (size_t)kMaxNodes - B)
        return PLB_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return PLB_ERR_CUDA;
    BCK(cudaSetDevice(device));
    plb_batch *b = new plb_batch();
    b->device = device;
    b->precision = precision;
    b->K = check_every;
    b->keep_macros = keep_macros;
    b->max_samples = max_samples;
    b->elem = elem_of(precision);
    b->cta = bp->cta_threads ? bp->cta_threads : batch_default_cta(precision);
    b->ordering = bp->ordering;
    b->prefetch = bp->l2_prefetch > 0 || (bp->l2_prefetch == 0 && precision == PLB_FP64);
    /* L2 groups on request: a budget in KiB, or -1 for 60% of the L2.  They
     * pay for pools of samples that fit in L2 (FP32 pools of 64^3 and 96^3
     * packs step 1.1-1.14x faster); on the batched workload, whose time goes
     * to samples larger than L2, they gained 1% of device time and cost
     * more than that in graph building */
    if (bp->l2_group_kb > 0) {
        b->group_bytes = (size_t)bp->l2_group_kb * 1024;
    } else if (bp->l2_group_kb == -1) {
        int l2 = 0;
        if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device) == cudaSuccess && l2 > 0)
            b->group_bytes = (size_t)l2 * 3 / 5;
    }
    b->cap_blocks = (long long)((capacity_nodes + B - 1) / B);
    b->rest = b->cap_blocks * B;
    b->npad = b->rest + B;
    b->s.resize((size_t)max_samples);
    b->free_blocks[0] = b->cap_blocks;
    cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->adm, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    auto al = [&](auto **p, size_t bytes) {
        if (e == cudaSuccess) e = plb_cuda_malloc((void **)p, bytes ? bytes : 16);
        b->bytes += bytes;
    };
    const size_t np = (size_t)b->npad;
    al(&b->f[0], b->elem * Q * np);
    al(&b->f[1], b->elem * Q * np);
    al(&b->nbr, 4 * 18 * np);
    al(&b->perm, 4 * np);
    al(&b->coord, 2 * 3 * np);
    if (keep_macros) al(&b->macro, 8 * 4 * np);
    al(&b->blk, 4 * (size_t)b->cap_blocks);
    al(&b->blist, 4 * (size_t)b->cap_blocks);
    al(&b->sdev, sizeof(SampleDev) * (size_t)max_samples);
    al(&b->sactive, 4 * (size_t)max_samples);
    al(&b->partial, 8 * 3 * 2 * (size_t)b->cap_blocks);
    al(&b->ssum, 8 * 3 * (size_t)max_samples);
    al(&b->serr, 4 * (size_t)max_samples);
    al(&b->t_dev, 4);
    al(&b->dgroups, 4 * 2 * (size_t)max_samples);
    al(&b->gcur, 4);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&b->h_ssum, 8 * 3 * (size_t)max_samples);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&b->h_serr, 4 * (size_t)max_samples);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->blk, 0xff, 4 * (size_t)b->cap_blocks, b->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->sactive, 0, 4 * (size_t)max_samples, b->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->serr, 0, 4 * (size_t)max_samples, b->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->t_dev, 0, 4, b->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->partial, 0, 8 * 3 * 2 * (size_t)b->cap_blocks, b->st);
    if (e == cudaSuccess) {
        k_fill_rest<<<1, B, 0, b->st>>>(b->f[0], b->f[1], b->npad, b->rest, b->rest + 1,
                                        (int)b->elem);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) {
        fprintf(stderr, "porelb_gpu: batch create failed: %s\n", cudaGetErrorString(e));
        batch_free(b);
        return e == cudaErrorMemoryAllocation ? PLB_ERR_NOMEM : PLB_ERR_CUDA;
    }
    *out = b;
    return PLB_OK;
}

static long long alloc_blocks(plb_batch *b, long long nblk)
{
    for (auto it = b->free_blocks.begin(); it != b->free_blocks.end(); ++it) {
        if (it->second >= nblk) {
            const long long start = it->first, len = it->second;
            b->free_blocks.erase(it);
            if (len > nblk) b->free_blocks[start + nblk] = len - nblk;
            return start;
        }
    }
    return -1;
}

static void free_range(plb_batch *b, long long start, long long len)
{
    auto it = b->free_blocks.emplace(start, len).first;
    auto nx = std::next(it);
    if (nx != b->free_blocks.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        b->free_blocks.erase(nx);
    }
    if (it != b->free_blocks.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            b->free_blocks.erase(it);
        }
    }
}

/* A sample whose tables and state are in place joins the pool: at once
 * when no interval runs, else at the next launch (the interval in flight
 * must not see it). */
static void activate(plb_batch *b, int sid)
{
    SampleHost &h = b->s[sid];
    h.active = 1;
    h.pending = 1;
    b->list_dirty = true;
}

/* Admit a sample whose flag grid is on the device. */
static int add_dflag(plb_batch *b, const uint8_t *dflag, int nx, int ny, int nz,
                     const plb_sample_params *sp, int *id)
{
    int sid = -1;
    for (int k = 0; k < b->max_samples; k++)
        if (!b->s[k].used) { sid = k; break; }
    if (sid < 0) return PLB_ERR_NOMEM;
    const size_t cells = (size_t)nx * ny * nz;
    const size_t words = (cells + 31) / 32;
    uint32_t *lexbits = nullptr, *lexoffs = nullptr;
    int n = 0, slab0 = 0, rc = PLB_OK;
    long long blk0 = -1, nblk = 0;
    if (plb_cuda_malloc(&lexbits, words * 4) != cudaSuccess ||
        plb_cuda_malloc(&lexoffs, words * 4) != cudaSuccess)
        rc = PLB_ERR_NOMEM;
    if (rc == PLB_OK) rc = flag_rank(dflag, nx, ny, nz, 1, lexbits, lexoffs, &n, &slab0, b->adm);
    if (rc == PLB_OK) {
        nblk = (n + B - 1) / B;
        if (nblk == 0) nblk = 1;
        blk0 = alloc_blocks(b, nblk);
        if (blk0 < 0) rc = PLB_ERR_NOMEM;
    }
    if (rc == PLB_OK) {
        const long long base = blk0 * B;
        const int order = b->ordering == PLB_ORDER_AUTO
                              ? plb_auto_ordering(n, nz, (int)b->elem, b->device)
                              : b->ordering;
        rc = flag_tables(dflag, nx, ny, nz, 1, order, 0, 0, lexbits, lexoffs, n,
                         b->npad, b->perm + base, b->coord + base, b->nbr + base,
                         (uint32_t)base, (uint32_t)b->rest, b->adm);
        if (rc != PLB_OK) free_range(b, blk0, nblk);
    }
    cudaFree(lexbits);
    cudaFree(lexoffs);
    if (rc != PLB_OK) return rc;

    SampleHost &h = b->s[sid];
    h = SampleHost();
    h.used = 1;
    h.blk0 = blk0;
    h.nblk = nblk;
    h.n = n;
    h.nx = nx; h.ny = ny; h.nz = nz;
    h.tau = sp->tau;
    h.force = sp->force_x;
    h.tol = sp->tol;
    h.handoff_tol = sp->handoff_tol > sp->tol ? sp->handoff_tol : 0.0;
    h.max_steps = sp->max_steps > 0 ? sp->max_steps : (1LL << 40);
    h.nu = 1.0 / 3.0 * (sp->tau - 0.5);
    h.start = b->t;
    /* 16-bit deviations: scale so that the expected deviation after the
     * first interval (|g| ~ 3 F K) sits near 2^13; adapted after each check */
    h.scale = 1.f;
    if (b->precision == PLB_FP16DEV) {
        double g = 3.0 * fabs(sp->force_x) * b->K;
        if (g < 1e-6) g = 1e-6;
        h.scale = (float)exp2(floor(log2(8192.0 / g)));
        if (h.scale > 1e9f) h.scale = 1e9f;
    }
    SampleDev &d = h.dev;
    memset(&d, 0, sizeof(d));
    make_coeffs(sp->tau, sp->force_x, h.scale, &d.co);
    d.base = blk0 * B;
    d.n = n;
    /* a sample admitted while an interval runs starts after it */
    d.start = (int)(b->t + (b->in_flight ? b->K : 0));
    h.start = d.start;
    BCK(cudaMemcpyAsync(b->sdev + sid, &d, sizeof(d), cudaMemcpyHostToDevice, b->adm));
    BCK(cudaMemsetAsync(b->serr + sid, 0, 4, b->adm));
    if (n > 0)
        k_fill_rest<<<gb(n, B), B, 0, b->adm>>>(b->f[0], b->f[1], b->npad, d.base, d.base + n,
                                               (int)b->elem);
    k_set_blocks<<<gb(nblk, B), B, 0, b->adm>>>(b->blk, blk0, nblk, sid, n);
    BCK(cudaGetLastError());
    BCK(cudaStreamSynchronize(b->adm));
    activate(b, sid);
    *id = sid;
    return PLB_OK;
}

int plb_batch_add_flag(plb_batch *b, const uint8_t *flag, int nx, int ny, int nz,
                       const plb_sample_params *sp, int *id)
{
    if (!b || !flag || !sp || !id || nx <= 0 || ny <= 0 || nz <= 0 || nx > 65536 ||
        ny > 65536 || nz > 65536 || !(sp->tau > 0.5))
        return PLB_ERR_ARG;
    BCK(cudaSetDevice(b->device));
    const size_t cells = (size_t)nx * ny * nz;
    uint8_t *d = nullptr;
    BCK(plb_cuda_malloc(&d, cells));
    int rc = PLB_OK;
    if (cudaMemcpyAsync(d, flag, cells, cudaMemcpyHostToDevice, b->adm) != cudaSuccess)
        rc = PLB_ERR_CUDA;
    if (rc == PLB_OK) rc = add_dflag(b, d, nx, ny, nz, sp, id);
    cudaStreamSynchronize(b->adm);
    cudaFree(d);
    return rc;
}

int plb_batch_add_packed(plb_batch *b, uint64_t seed, int nx, int ny, int nz,
                         double rmin, double rmax, double porosity,
                         const plb_sample_params *sp, int *id, int *num_spheres,
                         double *porosity_out)
{
    if (!b || !sp || !id || nx <= 0 || ny <= 0 || nz <= 0 || nx > 65536 ||
        ny > 65536 || nz > 65536 || !(sp->tau > 0.5) || !(rmin > 0.0) || rmax < rmin ||
        !(porosity >= 0.0) || !(porosity <= 1.0))
        return PLB_ERR_ARG;
    BCK(cudaSetDevice(b->device));
    const size_t cells = (size_t)nx * ny * nz;
    uint8_t *d = nullptr;
    BCK(plb_cuda_malloc(&d, cells));
    int rc = sphere_pack_device(seed, nx, ny, nz, rmin, rmax, porosity, d, num_spheres,
                                porosity_out, b->adm);
    if (rc == PLB_OK) rc = add_dflag(b, d, nx, ny, nz, sp, id);
    cudaStreamSynchronize(b->adm);
    cudaFree(d);
    return rc;
}

/* A chain of K batch-step kernel nodes (the last writes the sums) from
 * buffer cur, over `grid` CTAs; with `grouped` the launches step the L2
 * group *gcur and a last node moves *gcur to the next group. */
static cudaError_t step_chain(plb_batch *b, bool grouped, int grid,
                              std::vector<BatchArgs> &args,
                              std::vector<cudaGraphNode_t> &nodes, cudaGraph_t *out)
{
    BatchArgs a;
    memset(&a, 0, sizeof(a));
    a.nbr = b->nbr;
    a.npad = b->npad;
    a.blk_list = b->blist;
    /* prefetch the pool block half a wave of CTAs ahead (FP64 by default) */
    a.pf_blocks = b->prefetch ? (batch_wave_blocks(b->precision, b->cta) + 1) / 2 : 0;
    const int h = B / b->cta;
    a.part_stride = h * b->cap_blocks;
    a.blk_sample = b->blk;
    a.samples = b->sdev;
    a.t_base = b->t_dev;
    a.macro = b->macro;
    a.partial = b->partial;
    a.serr = b->serr;
    if (grouped) {
        a.grp = b->dgroups;
        a.grp_cur = b->gcur;
    }
    const int bt = b->cta;
    const void *fn = batch_step_kernel(b->precision, false, bt);
    const void *fn_m = batch_step_kernel(b->precision, true, bt);
    args.assign((size_t)b->K, a);
    nodes.assign((size_t)b->K, nullptr);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    cudaGraphNode_t prev = nullptr;
    int cur = b->cur;
    for (int k = 0; k < b->K && e == cudaSuccess; k++) {
        BatchArgs &ak = args[(size_t)k];
        ak.fin = b->f[cur];
        ak.fout = b->f[cur ^ 1];
        ak.t_off = k;
        cur ^= 1;
        void *kp[1] = {&ak};
        cudaKernelNodeParams p;
        memset(&p, 0, sizeof(p));
        p.func = (void *)(k == b->K - 1 ? fn_m : fn);
        p.gridDim = dim3((unsigned)(grid > 0 ? grid : 1));
        p.blockDim = dim3((unsigned)bt);
        p.kernelParams = kp;
        e = cudaGraphAddKernelNode(&nodes[(size_t)k], g, prev ? &prev : nullptr,
                                   prev ? 1 : 0, &p);
        prev = nodes[(size_t)k];
    }
    if (grouped && e == cudaSuccess) {
        int *gc = b->gcur;
        int one = 1;
        void *kp[2] = {&gc, &one};
        cudaKernelNodeParams p;
        memset(&p, 0, sizeof(p));
        p.func = (void *)k_advance;
        p.gridDim = dim3(1);
        p.blockDim = dim3(1);
        p.kernelParams = kp;
        cudaGraphNode_t n = nullptr;
        e = cudaGraphAddKernelNode(&n, g, &prev, 1, &p);
    }
    if (e != cudaSuccess && g) {
        cudaGraphDestroy(g);
        g = nullptr;
    }
    *out = g;
    return e;
}

/* Build the interval graphs: the K-step chain over the samples outside the
 * L2 groups, the K-step chain of one group (replayed once per group), and
 * the tail: the step counter advance, the per-sample reduction and its
 * read-back.  The chains' grid follows the active list; when it changes
 * only the grid is updated (set_graph_grid), so admissions and retirements
 * never rebuild the graphs. */
static int build_graph(plb_batch *b)
{
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->gexec_grp) cudaGraphExecDestroy(b->gexec_grp);
    if (b->graph_grp) cudaGraphDestroy(b->graph_grp);
    if (b->gexec_tail) cudaGraphExecDestroy(b->gexec_tail);
    b->gexec = b->gexec_grp = b->gexec_tail = nullptr;
    b->graph = b->graph_grp = nullptr;
    const int h = B / b->cta;
    b->graph_grid = b->big_blocks * h;
    b->grp_grid = b->group_blocks_max * h;
    cudaError_t e = step_chain(b, false, b->graph_grid, b->step_args, b->step_nodes, &b->graph);
    if (e == cudaSuccess)
        e = step_chain(b, true, b->grp_grid, b->grp_args, b->grp_nodes, &b->graph_grp);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->gexec, b->graph, 0);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->gexec_grp, b->graph_grp, 0);
    cudaGraph_t tail = nullptr;
    if (e == cudaSuccess) e = cudaGraphCreate(&tail, 0);
    cudaGraphNode_t prev = nullptr;
    int *t_dev = b->t_dev;
    int K = b->K;
    if (e == cudaSuccess) {
        void *kp[2] = {&t_dev, &K};
        cudaKernelNodeParams p;
        memset(&p, 0, sizeof(p));
        p.func = (void *)k_advance;
        p.gridDim = dim3(1);
        p.blockDim = dim3(1);
        p.kernelParams = kp;
        e = cudaGraphAddKernelNode(&prev, tail, nullptr, 0, &p);
    }
    const SampleDev *sd = b->sdev;
    const int *sa = b->sactive;
    const double *part = b->partial;
    int nrows = (int)(h * b->cap_blocks);
    int hh = h;
    double *ssum = b->ssum;
    if (e == cudaSuccess) {
        void *kp[6] = {(void *)&sd, (void *)&sa, (void *)&part, &nrows, &hh, &ssum};
        cudaKernelNodeParams p;
        memset(&p, 0, sizeof(p));
        p.func = (void *)k_sample_sums;
        p.gridDim = dim3((unsigned)b->max_samples);
        p.blockDim = dim3(128);
        p.kernelParams = kp;
        cudaGraphNode_t n = nullptr;
        e = cudaGraphAddKernelNode(&n, tail, &prev, 1, &p);
        prev = n;
    }
    if (e == cudaSuccess) {
        cudaGraphNode_t n = nullptr;
        e = cudaGraphAddMemcpyNode1D(&n, tail, &prev, 1, b->h_ssum, b->ssum,
                                     8 * 3 * (size_t)b->max_samples, cudaMemcpyDeviceToHost);
        prev = n;
    }
    if (e == cudaSuccess) {
        cudaGraphNode_t n = nullptr;
        e = cudaGraphAddMemcpyNode1D(&n, tail, &prev, 1, b->h_serr, b->serr,
                                     4 * (size_t)b->max_samples, cudaMemcpyDeviceToHost);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->gexec_tail, tail, 0);
    if (tail) cudaGraphDestroy(tail);
    if (e != cudaSuccess) {
        fprintf(stderr, "porelb_gpu: batch graph build failed: %s\n", cudaGetErrorString(e));
        return PLB_ERR_CUDA;
    }
    b->graph_cur = b->cur;
    return PLB_OK;
}

/* Set the grid of the step nodes of one chain. */
static int set_chain_grid(plb_batch *b, cudaGraphExec_t exec, std::vector<BatchArgs> &args,
                          std::vector<cudaGraphNode_t> &nodes, int grid)
{
    const int bt = b->cta;
    const void *fn = batch_step_kernel(b->precision, false, bt);
    const void *fn_m = batch_step_kernel(b->precision, true, bt);
    for (int k = 0; k < b->K; k++) {
        void *kp[1] = {&args[(size_t)k]};
        cudaKernelNodeParams p;
        memset(&p, 0, sizeof(p));
        p.func = (void *)(k == b->K - 1 ? fn_m : fn);
        p.gridDim = dim3((unsigned)grid);
        p.blockDim = dim3((unsigned)bt);
        p.kernelParams = kp;
        BCK(cudaGraphExecKernelNodeSetParams(exec, nodes[(size_t)k], &p));
    }
    return PLB_OK;
}

/* The chains of the instantiated graphs get the current block counts as
 * their grids: the samples outside the groups, and the largest group. */
static int set_graph_grid(plb_batch *b)
{
    const int h = B / b->cta;
    const int grid = b->big_blocks * h;
    if (grid != b->graph_grid && grid > 0) {
        const int rc = set_chain_grid(b, b->gexec, b->step_args, b->step_nodes, grid);
        if (rc != PLB_OK) return rc;
        b->graph_grid = grid;
    }
    const int ggrid = b->group_blocks_max * h;
    if (ggrid != b->grp_grid && ggrid > 0) {
        const int rc = set_chain_grid(b, b->gexec_grp, b->grp_args, b->grp_nodes, ggrid);
        if (rc != PLB_OK) return rc;
        b->grp_grid = ggrid;
    }
    return PLB_OK;
}

/* The active pool blocks in the order the interval steps them: first the
 * samples that step outside the L2 groups, then the groups.  Samples whose
 * working set fits group_bytes are packed first fit, largest first, into
 * groups of at most group_bytes; since one chain with the largest group's
 * grid steps every group, a group below half the largest one's blocks
 * (mostly empty CTAs) steps with the samples outside the groups instead. */
static void order_blocks(plb_batch *b)
{
    std::vector<std::pair<long long, int>> order;
    for (int sid = 0; sid < b->max_samples; sid++)
        if (b->s[sid].active) order.emplace_back(b->s[sid].blk0, sid);
    std::sort(order.begin(), order.end());
    const size_t per_block = (size_t)B * (2 * Q * b->elem + 72);
    std::vector<int> small;
    std::vector<char> grouped((size_t)b->max_samples, 0);
    if (b->group_bytes > 0)
        for (auto &o : order)
            if ((size_t)b->s[o.second].nblk * per_block <= b->group_bytes)
                small.push_back(o.second);
    std::stable_sort(small.begin(), small.end(), [&](int x, int y) {
        return b->s[x].nblk > b->s[y].nblk;
    });
    std::vector<std::vector<int>> bins;
    std::vector<size_t> used;
    for (int sid : small) {
        const size_t need = (size_t)b->s[sid].nblk * per_block;
        size_t k = 0;
        while (k < bins.size() && used[k] + need > b->group_bytes) k++;
        if (k == bins.size()) {
            bins.emplace_back();
            used.push_back(0);
        }
        bins[k].push_back(sid);
        used[k] += need;
    }
    size_t biggest = 0;
    for (size_t u : used) biggest = std::max(biggest, u);
    for (size_t k = 0; k < bins.size(); k++)
        if (2 * used[k] >= biggest)
            for (int sid : bins[k]) grouped[(size_t)sid] = 1;
    b->hlist.clear();
    b->hgroups.clear();
    for (auto &o : order) {
        const SampleHost &h = b->s[o.second];
        if (grouped[(size_t)o.second]) continue;
        for (long long k = 0; k < h.nblk; k++) b->hlist.push_back((int)(h.blk0 + k));
    }
    b->big_blocks = (int)b->hlist.size();
    b->group_blocks_max = 0;
    for (size_t k = 0; k < bins.size(); k++) {
        if (2 * used[k] < biggest) continue;
        std::vector<int> members = bins[k];
        std::sort(members.begin(), members.end(),
                  [&](int x, int y) { return b->s[x].blk0 < b->s[y].blk0; });
        const int first = (int)b->hlist.size();
        for (int sid : members)
            for (long long q = 0; q < b->s[sid].nblk; q++)
                b->hlist.push_back((int)(b->s[sid].blk0 + q));
        const int cnt = (int)b->hlist.size() - first;
        b->hgroups.push_back(first);
        b->hgroups.push_back(cnt);
        b->group_blocks_max = std::max(b->group_blocks_max, cnt);
    }
}

/* The sample stops being stepped: it leaves the active list and its
 * blocks are freed (or, parked at the handoff tolerance, kept until it is
 * released). */
static void retire(plb_batch *b, int sid, int status, bool keep_blocks = false)
{
    SampleHost &h = b->s[sid];
    h.active = 0;
    h.finished = 1;
    h.status = status;
    h.parked = keep_blocks ? 1 : 0;
    const int zero = 0;
    cudaMemcpyAsync(b->sactive + sid, &zero, 4, cudaMemcpyHostToDevice, b->st);
    if (!keep_blocks) {
        k_set_blocks<<<gb(h.nblk, B), B, 0, b->st>>>(b->blk, h.blk0, h.nblk, -1, 0);
        free_range(b, h.blk0, h.nblk);
    }
    b->list_dirty = true;
    b->done.push_back(sid);
}

int plb_batch_launch(plb_batch *b, int *n_active)
{
    if (!b) return PLB_ERR_ARG;
    if (b->in_flight) return PLB_ERR_STATE;
    BCK(cudaSetDevice(b->device));
    int act = 0;
    for (auto &h : b->s) act += h.active;
    if (n_active) *n_active = act;
    if (act == 0) return PLB_OK;
    /* samples admitted since the last launch join now */
    const int one = 1;
    for (int sid = 0; sid < b->max_samples; sid++) {
        SampleHost &h = b->s[sid];
        if (h.pending) {
            BCK(cudaMemcpyAsync(b->sactive + sid, &one, 4, cudaMemcpyHostToDevice, b->st));
            h.pending = 0;
        }
        h.stepping = h.active;
    }
    if (b->list_dirty) {
        order_blocks(b);
        if (!b->hlist.empty())
            BCK(cudaMemcpyAsync(b->blist, b->hlist.data(), 4 * b->hlist.size(),
                                cudaMemcpyHostToDevice, b->st));
        if (!b->hgroups.empty())
            BCK(cudaMemcpyAsync(b->dgroups, b->hgroups.data(), 4 * b->hgroups.size(),
                                cudaMemcpyHostToDevice, b->st));
        b->list_dirty = false;
    }
    if (!b->gexec || b->graph_cur != b->cur) {
        int rc = build_graph(b);
        if (rc != PLB_OK) return rc;
    } else {
        int rc = set_graph_grid(b);
        if (rc != PLB_OK) return rc;
    }
    BCK(cudaEventRecord(b->ev0, b->st));
    if (b->big_blocks > 0) BCK(cudaGraphLaunch(b->gexec, b->st));
    const int ngroups = (int)(b->hgroups.size() / 2);
    if (ngroups > 0) {
        BCK(cudaMemsetAsync(b->gcur, 0, 4, b->st));
        for (int g = 0; g < ngroups; g++) BCK(cudaGraphLaunch(b->gexec_grp, b->st));
    }
    BCK(cudaGraphLaunch(b->gexec_tail, b->st));
    BCK(cudaEventRecord(b->ev1, b->st));
    b->in_flight = true;
    return PLB_OK;
}

int plb_batch_finish(plb_batch *b)
{
    if (!b) return PLB_ERR_ARG;
    if (!b->in_flight) return PLB_OK;
    BCK(cudaSetDevice(b->device));
    BCK(cudaStreamSynchronize(b->st));
    b->in_flight = false;
    if (cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1) != cudaSuccess) b->last_ms = 0.f;
    b->t += b->K;
    /* K is even: the ping-pong parity is back where it started */
    for (int sid = 0; sid < b->max_samples; sid++) {
        SampleHost &h = b->s[sid];
        if (!h.stepping) continue;
        h.stepping = 0;
        h.steps = b->t - h.start;
        const double sux = b->h_ssum[3 * sid];
        const double cells = (double)h.nx * h.ny * h.nz;
        h.prev_ux = h.ux;
        h.ux = sux / cells;
        h.mass = b->h_ssum[3 * sid + 1];
        h.k_darcy = h.force != 0.0 ? h.ux * h.nu / h.force : 0.0;
        h.checks++;
        const unsigned err = b->h_serr[sid];
        if (err & 4u) { retire(b, sid, PLB_ERR_DENSITY); continue; }
        if (err & 1u) { retire(b, sid, PLB_ERR_STATE); continue; }
        const double change = fabs(h.ux - h.prev_ux);
        if (h.checks >= 2 && h.ux != 0.0 && change <= h.tol * fabs(h.ux)) {
            retire(b, sid, 1);
            continue;
        }
        if (h.steps >= h.max_steps) { retire(b, sid, 2); continue; }
        if (h.checks >= 2 && h.ux != 0.0 && h.handoff_tol > 0.0 &&
            change <= h.handoff_tol * fabs(h.ux)) {
            retire(b, sid, 4, true);
            continue;
        }
        /* 16-bit deviations: keep the largest stored value near 2^13-2^14 */
        if (b->precision == PLB_FP16DEV) {
            const double big = b->h_ssum[3 * sid + 2];
            float factor = 1.f;
            if (big > 16384.0) factor = 0.25f;
            else if (big > 0.0 && big < 2048.0 && h.scale < 1e9f) factor = 4.f;
            if (factor != 1.f) {
                const long long base = h.blk0 * B;
                k_rescale<__half><<<gb(h.n, B), B, 0, b->st>>>((__half *)b->f[b->cur], b->npad,
                                                              base, base + h.n, factor);
                h.scale *= factor;
                h.dev.co.scale = h.scale;
                h.dev.co.inv_scale = 1.0f / h.scale;
                BCK(cudaMemcpyAsync(b->sdev + sid, &h.dev, sizeof(SampleDev),
                                    cudaMemcpyHostToDevice, b->st));
            }
        }
    }
    BCK(cudaStreamSynchronize(b->st));
    return PLB_OK;
}

int plb_batch_run(plb_batch *b, int intervals, int *n_active)
{
    if (!b || intervals < 0) return PLB_ERR_ARG;
    for (int r = 0; r < intervals; r++) {
        int act = 0;
        int rc = plb_batch_launch(b, &act);
        if (rc != PLB_OK) return rc;
        if (act == 0) break;
        rc = plb_batch_finish(b);
        if (rc != PLB_OK) return rc;
    }
    if (n_active) {
        int act = 0;
        for (auto &h : b->s) act += h.active;
        *n_active = act;
    }
    return PLB_OK;
}

static bool dev_form(int precision)
{
    return precision == PLB_FP32 || precision == PLB_FP16DEV || precision == PLB_BF16DEV;
}

template <typename TI>
static void convert_to(const plb_batch *src, const SampleHost &hs, plb_batch *dst,
                       long long db, float scale_out)
{
    const TI *in = (const TI *)src->f[src->cur];
    const long long sb = hs.blk0 * B;
    const float inv = 1.0f / hs.scale;
    switch (dst->precision) {
    case PLB_FP32:
        k_convert_dev<TI, float><<<gb(hs.n, B), B, 0, dst->adm>>>(
            in, src->npad, sb, inv, (float *)dst->f[dst->cur], dst->npad, db, scale_out, hs.n);
        break;
    case PLB_FP16DEV:
        k_convert_dev<TI, __half><<<gb(hs.n, B), B, 0, dst->adm>>>(
            in, src->npad, sb, inv, (__half *)dst->f[dst->cur], dst->npad, db, scale_out, hs.n);
        break;
    default:
        k_convert_dev<TI, __nv_bfloat16><<<gb(hs.n, B), B, 0, dst->adm>>>(
            in, src->npad, sb, inv, (__nv_bfloat16 *)dst->f[dst->cur], dst->npad, db,
            scale_out, hs.n);
        break;
    }
}

int plb_batch_transfer(plb_batch *src, int id, plb_batch *dst, int *new_id)
{
    if (!src || !dst || src == dst || !new_id || id < 0 || id >= src->max_samples)
        return PLB_ERR_ARG;
    const SampleHost &hs = src->s[id];
    if (!hs.used || !hs.parked) return PLB_ERR_STATE;
    if (src->device != dst->device || src->K != dst->K || !dev_form(src->precision) ||
        !dev_form(dst->precision))
        return PLB_ERR_ARG;
    BCK(cudaSetDevice(dst->device));
    int sid = -1;
    for (int k = 0; k < dst->max_samples; k++)
        if (!dst->s[k].used) { sid = k; break; }
    if (sid < 0) return PLB_ERR_NOMEM;
    const long long blk0 = alloc_blocks(dst, hs.nblk);
    if (blk0 < 0) return PLB_ERR_NOMEM;
    const long long sb = hs.blk0 * B, db = blk0 * B;
    const int n = hs.n;
    /* the 16-bit target keeps the source's scale, or takes one that puts
     * the largest deviation near 2^13 */
    float scale = 1.f;
    if (dst->precision == PLB_FP16DEV) {
        if (src->precision == PLB_FP16DEV) {
            scale = hs.scale;
        } else {
            double g = 3.0 * fabs(hs.force) * dst->K;
            if (g < 1e-6) g = 1e-6;
            scale = (float)exp2(floor(log2(8192.0 / g)));
            if (scale > 1e9f) scale = 1e9f;
        }
    }
    cudaError_t e = cudaSuccess;
    if (n > 0) {
        e = cudaMemcpyAsync(dst->perm + db, src->perm + sb, 4 * (size_t)n,
                            cudaMemcpyDeviceToDevice, dst->adm);
        for (int r = 0; r < 3 && e == cudaSuccess; r++)
            e = cudaMemcpyAsync(dst->coord + r * dst->npad + db, src->coord + r * src->npad + sb,
                                2 * (size_t)n, cudaMemcpyDeviceToDevice, dst->adm);
        if (e == cudaSuccess) {
            k_translate_words<<<gb(n, B), B, 0, dst->adm>>>(src->nbr, src->npad, sb,
                                                           (uint32_t)src->rest, dst->nbr,
                                                           dst->npad, db, (uint32_t)dst->rest, n);
            switch (src->precision) {
            case PLB_FP32: convert_to<float>(src, hs, dst, db, scale); break;
            case PLB_FP16DEV: convert_to<__half>(src, hs, dst, db, scale); break;
            default: convert_to<__nv_bfloat16>(src, hs, dst, db, scale); break;
            }
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        free_range(dst, blk0, hs.nblk);
        fprintf(stderr, "porelb_gpu: batch transfer failed: %s\n", cudaGetErrorString(e));
        return PLB_ERR_CUDA;
    }
    SampleHost &h = dst->s[sid];
    h = hs;
    h.used = 1;
    h.active = 0;
    h.finished = 0;
    h.parked = 0;
    h.stepping = 0;
    h.pending = 0;
    h.status = 0;
    h.handoff_tol = 0.0;
    h.blk0 = blk0;
    h.scale = scale;
    /* the step count goes on from where the source pool stopped (the
     * it > 0 rule of porelb.c:347-348 counts from the sample's start) */
    h.start = dst->t + (dst->in_flight ? dst->K : 0) - hs.steps;
    SampleDev &d = h.dev;
    memset(&d, 0, sizeof(d));
    make_coeffs(h.tau, h.force, h.scale, &d.co);
    d.base = db;
    d.n = n;
    d.start = (int)h.start;
    BCK(cudaMemcpyAsync(dst->sdev + sid, &d, sizeof(d), cudaMemcpyHostToDevice, dst->adm));
    BCK(cudaMemsetAsync(dst->serr + sid, 0, 4, dst->adm));
    k_set_blocks<<<gb(hs.nblk, B), B, 0, dst->adm>>>(dst->blk, blk0, hs.nblk, sid, n);
    BCK(cudaGetLastError());
    BCK(cudaStreamSynchronize(dst->adm));
    activate(dst, sid);
    *new_id = sid;
    return PLB_OK;
}

int plb_batch_poll(plb_batch *b, int *ids, int max_ids, int *count)
{
    if (!b || !count || (max_ids > 0 && !ids)) return PLB_ERR_ARG;
    int c = 0;
    while (c < max_ids && !b->done.empty()) {
        ids[c++] = b->done.front();
        b->done.erase(b->done.begin());
    }
    *count = c;
    return PLB_OK;
}

int plb_batch_result(plb_batch *b, int id, double *k_darcy, double *mean_ux,
                     long long *steps, int *status)
{
    if (!b || id < 0 || id >= b->max_samples || !b->s[id].used) return PLB_ERR_ARG;
    const SampleHost &h = b->s[id];
    if (k_darcy) *k_darcy = h.k_darcy;
    if (mean_ux) *mean_ux = h.ux;
    if (steps) *steps = h.steps;
    if (status) *status = h.finished ? h.status : 0;
    return PLB_OK;
}

int plb_batch_release(plb_batch *b, int id)
{
    if (!b || id < 0 || id >= b->max_samples || !b->s[id].used) return PLB_ERR_ARG;
    /* a sample the interval in flight steps is released after it */
    if (b->s[id].stepping) return PLB_ERR_STATE;
    BCK(cudaSetDevice(b->device));
    if (b->s[id].active) retire(b, id, 3);
    if (b->s[id].parked) {
        SampleHost &h = b->s[id];
        k_set_blocks<<<gb(h.nblk, B), B, 0, b->adm>>>(b->blk, h.blk0, h.nblk, -1, 0);
        BCK(cudaGetLastError());
        BCK(cudaStreamSynchronize(b->adm));
        free_range(b, h.blk0, h.nblk);
        h.parked = 0;
    }
    BCK(cudaStreamSynchronize(b->st));
    for (auto it = b->done.begin(); it != b->done.end();)
        it = (*it == id) ? b->done.erase(it) : std::next(it);
    b->s[id] = SampleHost();
    return PLB_OK;
}

int plb_batch_get_f(plb_batch *b, int id, double *f_aos)
{
    if (!b || id < 0 || id >= b->max_samples || !(b->s[id].active || b->s[id].parked) ||
        !f_aos)
        return PLB_ERR_ARG;
    if (b->in_flight) return PLB_ERR_STATE;
    BCK(cudaSetDevice(b->device));
    const SampleHost &h = b->s[id];
    if (h.n == 0) return PLB_OK;
    double *d = nullptr;
    const size_t bytes = 8 * Q * (size_t)h.n;
    BCK(plb_cuda_malloc(&d, bytes));
    const long long base = h.blk0 * B;
    const float inv = 1.0f / h.scale;
    const void *f = b->f[b->cur];
    switch (b->elem) {
    case 8: k_get_f_sample<double><<<gb(h.n, B), B, 0, b->st>>>((const double *)f, b->npad, base, h.n, b->perm, inv, d); break;
    case 4: k_get_f_sample<float><<<gb(h.n, B), B, 0, b->st>>>((const float *)f, b->npad, base, h.n, b->perm, inv, d); break;
    default:
        if (b->precision == PLB_FP16DEV)
            k_get_f_sample<__half><<<gb(h.n, B), B, 0, b->st>>>((const __half *)f, b->npad, base, h.n, b->perm, inv, d);
        else
            k_get_f_sample<__nv_bfloat16><<<gb(h.n, B), B, 0, b->st>>>((const __nv_bfloat16 *)f, b->npad, base, h.n, b->perm, inv, d);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(f_aos, d, bytes, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    cudaFree(d);
    return e == cudaSuccess ? PLB_OK : PLB_ERR_CUDA;
}

int plb_batch_get_macros(plb_batch *b, int id, double *rho, double *ux,
                         double *uy, double *uz)
{
    if (!b || id < 0 || id >= b->max_samples || !b->s[id].active || !b->macro)
        return PLB_ERR_ARG;
    if (b->in_flight) return PLB_ERR_STATE;
    BCK(cudaSetDevice(b->device));
    const SampleHost &h = b->s[id];
    if (h.n == 0) return PLB_OK;
    double *d = nullptr;
    BCK(plb_cuda_malloc(&d, 8 * 4 * (size_t)h.n));
    k_get_macro_sample<<<gb(h.n, B), B, 0, b->st>>>(b->macro, b->npad, h.blk0 * B, h.n,
                                                   b->perm, d);
    double *dst[4] = {rho, ux, uy, uz};
    cudaError_t e = cudaGetLastError();
    for (int c = 0; c < 4 && e == cudaSuccess; c++)
        if (dst[c])
            e = cudaMemcpyAsync(dst[c], d + (size_t)c * h.n, 8 * (size_t)h.n,
                                cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    cudaFree(d);
    return e == cudaSuccess ? PLB_OK : PLB_ERR_CUDA;
}

int plb_batch_info(plb_batch *b, long long *t, int *active, long long *used_nodes,
                   long long *capacity_nodes, size_t *device_bytes)
{
    if (!b) return PLB_ERR_ARG;
    int act = 0;
    long long used = 0;
    for (auto &h : b->s)
        if (h.active) {
            act++;
            used += h.nblk * B;
        }
    if (t) *t = b->t;
    if (active) *active = act;
    if (used_nodes) *used_nodes = used;
    if (capacity_nodes) *capacity_nodes = b->cap_blocks * B;
    if (device_bytes) *device_bytes = b->bytes;
    return PLB_OK;
}

int plb_batch_free_nodes(plb_batch *b, long long *largest_range, long long *total)
{
    if (!b) return PLB_ERR_ARG;
    long long big = 0, all = 0;
    for (const auto &r : b->free_blocks) {
        big = std::max(big, r.second);
        all += r.second;
    }
    int slots = 0;
    for (const auto &h : b->s) slots += !h.used;
    if (largest_range) *largest_range = slots > 0 ? big * B : 0;
    if (total) *total = all * B;
    return PLB_OK;
}

int plb_batch_interval_ms(plb_batch *b, float *ms)
{
    if (!b || !ms) return PLB_ERR_ARG;
    *ms = b->last_ms;
    return PLB_OK;
}

int plb_batch_sample_nodes(plb_batch *b, int id, int *num_node)
{
    if (!b || id < 0 || id >= b->max_samples || !b->s[id].used || !num_node)
        return PLB_ERR_ARG;
    *num_node = b->s[id].n;
    return PLB_OK;
}

void *plb_batch_stream(plb_batch *b) { return b ? (void *)b->st : nullptr; }
