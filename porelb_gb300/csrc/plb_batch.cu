/*
 * plb_batch.cu - many independent porous samples in one device pool.
 *
 * Samples of uneven size are concatenated as 256-node block ranges of one
 * node pool; a per-block map names the sample whose tau, force and storage
 * scale the step applies (k_batch_step, plb_step.cu).  All samples advance
 * together: one launch per lattice step covers every active block, and an
 * interval of K steps (the last writing the per-block sums) plus the
 * per-sample reduction is captured once in a CUDA graph and replayed.
 * After each interval the host checks each sample's steady-state criterion
 * (relative change of the mean u_x over the interval), retires converged
 * samples and frees their blocks; new samples are admitted at interval
 * boundaries into free block ranges (first fit).  A sample's arithmetic does
 * not depend on what else is in the pool, so its result is the same alone
 * and in a mix.
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

struct SampleHost {
    int used = 0, active = 0, finished = 0;
    long long blk0 = 0, nblk = 0;
    int n = 0, nx = 0, ny = 0, nz = 0;
    double tau = 0, force = 0, tol = 0, nu = 0;
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
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    long long graph_n = -1;
    int graph_cur = -1;
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
    delete b;
}

void plb_batch_destroy(plb_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->st) cudaStreamSynchronize(b->st);
    batch_free(b);
}

int plb_batch_create(size_t capacity_nodes, int max_samples, int precision,
                     int check_every, int keep_macros, int device,
                     plb_batch **out)
{
    if (!out) return PLB_ERR_ARG;
    *out = nullptr;
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
    b->cap_blocks = (long long)((capacity_nodes + B - 1) / B);
    b->rest = b->cap_blocks * B;
    b->npad = b->rest + B;
    b->s.resize((size_t)max_samples);
    b->free_blocks[0] = b->cap_blocks;
    cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    auto al = [&](auto **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc((void **)p, bytes ? bytes : 16);
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
    if (cudaMalloc(&lexbits, words * 4) != cudaSuccess ||
        cudaMalloc(&lexoffs, words * 4) != cudaSuccess)
        rc = PLB_ERR_NOMEM;
    if (rc == PLB_OK) rc = flag_rank(dflag, nx, ny, nz, 1, lexbits, lexoffs, &n, &slab0, b->st);
    if (rc == PLB_OK) {
        nblk = (n + B - 1) / B;
        if (nblk == 0) nblk = 1;
        blk0 = alloc_blocks(b, nblk);
        if (blk0 < 0) rc = PLB_ERR_NOMEM;
    }
    if (rc == PLB_OK) {
        const long long base = blk0 * B;
        rc = flag_tables(dflag, nx, ny, nz, 1, PLB_ORDER_MORTON, 0, 0, lexbits, lexoffs, n,
                         b->npad, b->perm + base, b->coord + base, b->nbr + base,
                         (uint32_t)base, (uint32_t)b->rest, b->st);
        if (rc != PLB_OK) free_range(b, blk0, nblk);
    }
    cudaFree(lexbits);
    cudaFree(lexoffs);
    if (rc != PLB_OK) return rc;

    SampleHost &h = b->s[sid];
    h = SampleHost();
    h.used = 1;
    h.active = 1;
    h.blk0 = blk0;
    h.nblk = nblk;
    h.n = n;
    h.nx = nx; h.ny = ny; h.nz = nz;
    h.tau = sp->tau;
    h.force = sp->force_x;
    h.tol = sp->tol;
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
    d.start = (int)b->t;
    const int one = 1;
    BCK(cudaMemcpyAsync(b->sdev + sid, &d, sizeof(d), cudaMemcpyHostToDevice, b->st));
    BCK(cudaMemcpyAsync(b->sactive + sid, &one, 4, cudaMemcpyHostToDevice, b->st));
    BCK(cudaMemsetAsync(b->serr + sid, 0, 4, b->st));
    if (n > 0)
        k_fill_rest<<<gb(n, B), B, 0, b->st>>>(b->f[0], b->f[1], b->npad, d.base, d.base + n,
                                              (int)b->elem);
    k_set_blocks<<<gb(nblk, B), B, 0, b->st>>>(b->blk, blk0, nblk, sid, n);
    BCK(cudaGetLastError());
    BCK(cudaStreamSynchronize(b->st));
    b->list_dirty = true;
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
    BCK(cudaMalloc(&d, cells));
    int rc = PLB_OK;
    if (cudaMemcpyAsync(d, flag, cells, cudaMemcpyHostToDevice, b->st) != cudaSuccess)
        rc = PLB_ERR_CUDA;
    if (rc == PLB_OK) rc = add_dflag(b, d, nx, ny, nz, sp, id);
    cudaStreamSynchronize(b->st);
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
    BCK(cudaMalloc(&d, cells));
    int rc = sphere_pack_device(seed, nx, ny, nz, rmin, rmax, porosity, d, num_spheres,
                                porosity_out, b->st);
    if (rc == PLB_OK) rc = add_dflag(b, d, nx, ny, nz, sp, id);
    cudaStreamSynchronize(b->st);
    cudaFree(d);
    return rc;
}

/* Capture one interval: K steps (the last writes the sums), the step
 * counter advance, the per-sample reduction and its read-back. */
static int build_graph(plb_batch *b)
{
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    const int nb = (int)b->hlist.size();
    BCK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    BatchArgs a;
    memset(&a, 0, sizeof(a));
    a.nbr = b->nbr;
    a.npad = b->npad;
    a.blk_list = b->blist;
    /* the FP64 form prefetches the pool block half a wave of CTAs ahead */
    a.pf_blocks = b->precision == PLB_FP64 ? (batch_wave_blocks(b->precision) + 1) / 2 : 0;
    const int h = batch_ctas_per_block(b->precision);
    a.part_stride = h * b->cap_blocks;
    a.blk_sample = b->blk;
    a.samples = b->sdev;
    a.t_base = b->t_dev;
    a.macro = b->macro;
    a.partial = b->partial;
    a.serr = b->serr;
    int cur = b->cur;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < b->K && e == cudaSuccess; k++) {
        a.fin = b->f[cur];
        a.fout = b->f[cur ^ 1];
        a.t_off = k;
        e = launch_batch_step(b->precision, k == b->K - 1, a, nb, b->st);
        cur ^= 1;
    }
    if (e == cudaSuccess) {
        k_advance<<<1, 1, 0, b->st>>>(b->t_dev, b->K);
        k_sample_sums<<<b->max_samples, 128, 0, b->st>>>(b->sdev, b->sactive, b->partial,
                                                         (int)(h * b->cap_blocks), h, b->ssum);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->h_ssum, b->ssum, 8 * 3 * (size_t)b->max_samples,
                            cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->h_serr, b->serr, 4 * (size_t)b->max_samples,
                            cudaMemcpyDeviceToHost, b->st);
    cudaError_t e2 = cudaStreamEndCapture(b->st, &b->graph);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->gexec, b->graph, 0);
    if (e != cudaSuccess) {
        fprintf(stderr, "porelb_gpu: batch graph capture failed: %s\n", cudaGetErrorString(e));
        return PLB_ERR_CUDA;
    }
    b->graph_n = nb;
    b->graph_cur = b->cur;
    return PLB_OK;
}

static void retire(plb_batch *b, int sid, int status)
{
    SampleHost &h = b->s[sid];
    h.active = 0;
    h.finished = 1;
    h.status = status;
    const int zero = 0;
    cudaMemcpyAsync(b->sactive + sid, &zero, 4, cudaMemcpyHostToDevice, b->st);
    k_set_blocks<<<gb(h.nblk, B), B, 0, b->st>>>(b->blk, h.blk0, h.nblk, -1, 0);
    free_range(b, h.blk0, h.nblk);
    b->list_dirty = true;
    b->done.push_back(sid);
}

int plb_batch_run(plb_batch *b, int intervals, int *n_active)
{
    if (!b || intervals < 0) return PLB_ERR_ARG;
    BCK(cudaSetDevice(b->device));
    for (int r = 0; r < intervals; r++) {
        int act = 0;
        for (auto &h : b->s) act += h.active;
        if (act == 0) break;
        if (b->list_dirty) {
            /* the pool blocks of the active samples, in pool order */
            std::vector<std::pair<long long, int>> order;
            for (int sid = 0; sid < b->max_samples; sid++)
                if (b->s[sid].active) order.emplace_back(b->s[sid].blk0, sid);
            std::sort(order.begin(), order.end());
            b->hlist.clear();
            for (auto &o : order) {
                const SampleHost &h = b->s[o.second];
                for (long long k = 0; k < h.nblk; k++) b->hlist.push_back((int)(h.blk0 + k));
            }
            if (!b->hlist.empty())
                BCK(cudaMemcpyAsync(b->blist, b->hlist.data(), 4 * b->hlist.size(),
                                    cudaMemcpyHostToDevice, b->st));
            b->list_dirty = false;
        }
        if (!b->gexec || b->graph_n != (long long)b->hlist.size() || b->graph_cur != b->cur) {
            int rc = build_graph(b);
            if (rc != PLB_OK) return rc;
        }
        BCK(cudaGraphLaunch(b->gexec, b->st));
        BCK(cudaStreamSynchronize(b->st));
        b->t += b->K;
        /* K is even: the ping-pong parity is back where it started */
        for (int sid = 0; sid < b->max_samples; sid++) {
            SampleHost &h = b->s[sid];
            if (!h.active) continue;
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
            if (h.checks >= 2 && h.ux != 0.0 &&
                fabs(h.ux - h.prev_ux) <= h.tol * fabs(h.ux)) {
                retire(b, sid, 1);
                continue;
            }
            if (h.steps >= h.max_steps) { retire(b, sid, 2); continue; }
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
                    BCK(cudaStreamSynchronize(b->st));
                }
            }
        }
        BCK(cudaStreamSynchronize(b->st));
    }
    if (n_active) {
        int act = 0;
        for (auto &h : b->s) act += h.active;
        *n_active = act;
    }
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
    BCK(cudaSetDevice(b->device));
    if (b->s[id].active) retire(b, id, 3);
    BCK(cudaStreamSynchronize(b->st));
    for (auto it = b->done.begin(); it != b->done.end();)
        it = (*it == id) ? b->done.erase(it) : std::next(it);
    b->s[id] = SampleHost();
    return PLB_OK;
}

int plb_batch_get_f(plb_batch *b, int id, double *f_aos)
{
    if (!b || id < 0 || id >= b->max_samples || !b->s[id].active || !f_aos)
        return PLB_ERR_ARG;
    BCK(cudaSetDevice(b->device));
    const SampleHost &h = b->s[id];
    if (h.n == 0) return PLB_OK;
    double *d = nullptr;
    const size_t bytes = 8 * Q * (size_t)h.n;
    BCK(cudaMalloc(&d, bytes));
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
    BCK(cudaSetDevice(b->device));
    const SampleHost &h = b->s[id];
    if (h.n == 0) return PLB_OK;
    double *d = nullptr;
    BCK(cudaMalloc(&d, 8 * 4 * (size_t)h.n));
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

int plb_batch_sample_nodes(plb_batch *b, int id, int *num_node)
{
    if (!b || id < 0 || id >= b->max_samples || !b->s[id].used || !num_node)
        return PLB_ERR_ARG;
    *num_node = b->s[id].n;
    return PLB_OK;
}

void *plb_batch_stream(plb_batch *b) { return b ? (void *)b->st : nullptr; }
