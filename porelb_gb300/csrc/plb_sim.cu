/*
 * plb_sim.cu - the solver handle: device-side table build (Morton order and
 * pull table), state management, macro/f readback, reductions.
 *
 * Replaces alloc_memory, check_V, init_para, build_send_recv_info,
 * init_dist_macro and the step loop of porelb.c:15-443.  The halo exchange
 * (porelb.c:143-312) has no counterpart: all rank slabs live in one device
 * memory and a cross-slab push is an ordinary pull through the table.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <atomic>

#include "plb_emu.h"
#include "plb_internal.h"

using namespace plb;

extern "C" void plb_host_constants(double tau, double force, double *omega,
                                   double *om1, double *k3, double *half_force,
                                   double *nu);

struct plb_sim {
    int n, nx, ny, nz, num_p;
    long long npad;
    int precision, ordering, halo, block, boundary, variant;
    int prefetch, wave; /* L2 prefetch on; resident blocks (0 = not queried) */
    int device;
    cudaStream_t stream;
    void *f[2];
    int cur;
    size_t elem;
    uint32_t *nbr;
    int *perm;        /* new -> reference index */
    uint16_t *coord;  /* [3][npad] x, y, z in new order */
    double *macro;    /* [4][npad] */
    double *partial;  /* [2][nblocks] */
    double *sums;     /* [2] */
    int nblocks;
    unsigned long long *err;
    unsigned int *flags;
    int *v_sub_start; /* host, num_p + 1 */
    double tau, omega, om1, k3, force, half_force, nu;
    fx::Consts fxk;
    float scale;
    int initialized, macro_valid;
    size_t dev_bytes;
    int err_it, err_node;
    int fallback_nodes_seen;
};

#define CK(call)                                                          \
    do {                                                                  \
        cudaError_t e_ = (call);                                          \
        if (e_ != cudaSuccess) {                                          \
            fprintf(stderr, "porelb_gpu: %s failed: %s (%s:%d)\n", #call, \
                    cudaGetErrorString(e_), __FILE__, __LINE__);          \
            return e_ == cudaErrorMemoryAllocation ? PLB_ERR_NOMEM        \
                                                   : PLB_ERR_CUDA;        \
        }                                                                 \
    } while (0)

/* ------------------------------------------------------ ordering */

int plb_auto_ordering(long long n, int nz, int elem_bytes, int device)
{
    /* bytes a step moves per node: 19 values in and out, 18 words, perm */
    const double bpn = 2.0 * 19 * elem_bytes + 72 + 4;
    int l2 = 0;
    if (nz <= 0 || cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device) != cudaSuccess ||
        l2 <= 0)
        return PLB_ORDER_MORTON;
    const double plane = bpn * (double)n / nz;
    /* measured: row order wins up to about 63 MB of such planes on a 126 MB
     * L2 (512^3 FP32) and loses from 105 MB (512^3 FP64, whose L2 prefetch
     * also takes room) */
    return 3.0 * plane <= 0.6 * (double)l2 ? PLB_ORDER_REFERENCE : PLB_ORDER_MORTON;
}

/* ------------------------------------------------------ allocation */

/* Device allocations made so far and the armed failure (0 = none): the
 * fault_at-th allocation after plb_fault_inject_alloc reports
 * cudaErrorMemoryAllocation without calling cudaMalloc. */
static std::atomic<long long> g_allocs{0};
static std::atomic<long long> g_fault_at{0};

cudaError_t plb_dev_malloc(void **p, size_t bytes)
{
    const long long k = ++g_allocs;
    const long long at = g_fault_at.load();
    if (at > 0 && k == at) {
        g_fault_at.store(0);
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes ? bytes : 16);
}

int plb_fault_inject_alloc(long long nth)
{
    g_fault_at.store(nth > 0 ? g_allocs.load() + nth : 0);
    return PLB_OK;
}

long long plb_alloc_count(void) { return g_allocs.load(); }

/* ---------------------------------------------------------------- scan */

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

/* exclusive scan of one tile of uint32 counts; tile total to sums[b] */
__global__ void __launch_bounds__(kScanThreads)
k_scan_tile(const uint32_t *in, uint32_t *out, uint32_t *sums, size_t m)
{
    __shared__ uint32_t warp_tot[32];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t t = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < m) ? in[base + k] : 0u;
        t += v[k];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t incl = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint32_t x = warp_tot[lane];
        uint32_t xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += y;
        }
        warp_tot[lane] = xi - x;
        if (lane == 31) sums[blockIdx.x] = xi;
    }
    __syncthreads();
    uint32_t run = warp_tot[wid] + incl - t;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < m) out[base + k] = run;
        run += v[k];
    }
}

/* exclusive scan of the tile sums, one block, in place */
__global__ void __launch_bounds__(kScanThreads)
k_scan_sums(uint32_t *sums, int ntiles)
{
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int b0 = 0; b0 < ntiles; b0 += kScanThreads) {
        const int k = b0 + threadIdx.x;
        const uint32_t t = k < ntiles ? sums[k] : 0u;
        uint32_t incl = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint32_t x = warp_tot[lane], xi = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, xi, o);
                if (lane >= o) xi += y;
            }
            warp_tot[lane] = xi - x;
        }
        __syncthreads();
        const uint32_t excl = carry + warp_tot[wid] + incl - t;
        __syncthreads();
        if (k < ntiles) sums[k] = excl;
        if (threadIdx.x == kScanThreads - 1) carry = excl + t;
        __syncthreads();
    }
}

__global__ void k_scan_add(uint32_t *out, const uint32_t *sums, size_t m)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) out[k] += sums[k / kScanTile];
}

static int exclusive_scan(const uint32_t *in, uint32_t *out, size_t m,
                          uint32_t *tmp, cudaStream_t s)
{
    const size_t ntiles = (m + kScanTile - 1) / kScanTile;
    if (ntiles > (size_t)0x7fffffff) return PLB_ERR_ARG;
    k_scan_tile<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, out, tmp, m);
    k_scan_sums<<<1, kScanThreads, 0, s>>>(tmp, (int)ntiles);
    k_scan_add<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(out, tmp, m);
    CK(cudaGetLastError());
    return PLB_OK;
}

namespace plb {
void make_coeffs(double tau, double force, float scale, Coeffs *c)
{
    memset(c, 0, sizeof(*c));
    plb_host_constants(tau, force, &c->omega, &c->om1, &c->k3, &c->half_force,
                       nullptr);
    c->force = force;
    c->omega_f = (float)c->omega;
    c->om1_f = (float)c->om1;
    c->c_f = (float)(c->k3 * force);
    c->half_force_f = (float)c->half_force;
    c->scale = scale;
    c->inv_scale = 1.0f / scale;
    c->fxk = fx::make_consts(tau, force);
    const double consts[5] = {c->omega, c->om1, c->k3, c->force, c->half_force};
    for (double x : consts) {
        uint64_t b;
        memcpy(&b, &x, 8);
        c->exact_native |= (int)emu::outside_node_range(b);
    }
}

int scan_words(const uint32_t *cnt, uint32_t *offs, size_t m, cudaStream_t st)
{
    const size_t ntiles = (m + kScanTile - 1) / kScanTile;
    uint32_t *tmp = nullptr;
    if (plb_cuda_malloc(&tmp, ntiles * 4 + 4) != cudaSuccess) return PLB_ERR_NOMEM;
    int rc = exclusive_scan(cnt, offs, m, tmp, st);
    cudaStreamSynchronize(st);
    cudaFree(tmp);
    return rc;
}
}  // namespace plb

/* --------------------------------------------------------- table build */

struct MortonBits {
    int bx, by, bz;
};

__host__ __device__ static inline uint64_t morton3(uint32_t x, uint32_t y,
                                                   uint32_t z, MortonBits b)
{
    uint64_t c = 0;
    int pos = 0;
    const int top = b.bx > b.by ? (b.bx > b.bz ? b.bx : b.bz) : (b.by > b.bz ? b.by : b.bz);
    for (int k = 0; k < top; k++) {
        if (k < b.bx) c |= (uint64_t)((x >> k) & 1u) << pos++;
        if (k < b.by) c |= (uint64_t)((y >> k) & 1u) << pos++;
        if (k < b.bz) c |= (uint64_t)((z >> k) & 1u) << pos++;
    }
    return c;
}

static int ceil_log2(int v)
{
    int b = 0;
    while ((1LL << b) < v) b++;
    return b;
}

/* error bits of the table build */
enum { kBadCoord = 1, kBadId = 2, kBadPid = 4, kDupCoord = 8 };

__global__ void k_morton_mark(const plb_node_info *V, int n, int nx, int ny,
                              int nz, MortonBits b, uint32_t *bitmap,
                              unsigned *bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const plb_node_info &r = V[i];
    if (r.x >= nx || r.y >= ny || r.z >= nz) {
        atomicOr(bad, kBadCoord);
        return;
    }
    const uint64_t c = morton3(r.x, r.y, r.z, b);
    atomicOr(bitmap + (c >> 5), 1u << (c & 31));
}

/* a node number the Morton numbering left unassigned: two records on one
 * cell */
__global__ void k_perm_holes(const int *perm, int n, unsigned *bad)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && perm[k] < 0) atomicOr(bad, kDupCoord);
}

__global__ void k_popc(const uint32_t *bitmap, uint32_t *cnt, size_t m)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) cnt[k] = __popc(bitmap[k]);
}

__global__ void k_morton_assign(const plb_node_info *V, int n, int nx, int ny,
                                int nz, MortonBits b, const uint32_t *bitmap,
                                const uint32_t *offs, int *perm, int *inv,
                                unsigned *bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const plb_node_info &r = V[i];
    if (r.x >= nx || r.y >= ny || r.z >= nz) return;
    const uint64_t c = morton3(r.x, r.y, r.z, b);
    const uint32_t word = bitmap[c >> 5];
    const int k = (int)(offs[c >> 5] + __popc(word & ((1u << (c & 31)) - 1u)));
    if (k < 0 || k >= n) {
        atomicOr(bad, kDupCoord);
        return;
    }
    if (atomicExch(perm + k, i) != -1) atomicOr(bad, kDupCoord);
    inv[i] = k;
}

__global__ void k_identity(int *perm, int *inv, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        perm[i] = i;
        inv[i] = i;
    }
}

/* Pull table: word for node k (new order), direction j.  The slot f1[x][j]
 * of the reference is written by the push of s = x - e_j if s is fluid
 * (stream_inner_nodes, porelb.c:293-295) and by the bounce-back of x if
 * t = x + e_j is solid (porelb.c:296-297).  nb_info[re(j)-1] describes s and
 * nb_info[j-1] describes t.  When both write, the later in the rank's node
 * order wins; a push from another rank arrives after the local stream
 * (update_recv_dist, porelb.c:433) and wins when remote_wins is set.  A slot
 * nobody writes keeps its initial value: it reads the rest slot n. */
__global__ void k_build_nbr(const plb_node_info *V, const int *perm,
                            const int *inv, const int *start, int num_p,
                            int n, long long npad, int remote_wins, int halfway,
                            uint32_t *nbr, uint16_t *coord, unsigned *bad)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = perm[k];
    if (i < 0 || i >= n) {
        atomicOr(bad, kDupCoord);
        return;
    }
    int lo = 0, hi = num_p - 1; /* rank of i: last p with start[p] <= i */
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    const int rank = lo;
    const plb_node_info &r = V[i];
    coord[k] = r.x;
    coord[npad + k] = r.y;
    coord[2 * npad + k] = r.z;
#pragma unroll
    for (int j = 1; j < Q; j++) {
        const plb_neighbor_info sn = r.nb_info[opp(j) - 1];
        const plb_neighbor_info tn = r.nb_info[j - 1];
        const bool push = sn.node_type != PLB_TYPE_SOLID;
        const bool bounce = tn.node_type == PLB_TYPE_SOLID;
        long long sg = -1;
        bool ext = false;
        if (push) {
            int q = rank;
            if (sn.node_type == PLB_TYPE_EXTERN) {
                q = sn.node_pid;
                ext = true;
                if (q >= num_p || q == rank) {
                    atomicOr(bad, kBadPid);
                    q = rank;
                }
            } else if (sn.node_type != PLB_TYPE_FLUID) {
                atomicOr(bad, kBadPid);
            }
            sg = (long long)start[q] + sn.node_id;
            if (sg >= start[q + 1]) {
                atomicOr(bad, kBadId);
                sg = i;
            }
        }
        uint32_t word;
        if (halfway)  /* standard rule: pull from s, or bounce if s is solid */
            word = push ? (uint32_t)inv[sg] : bounce_word(j, k, npad);
        else if (push && (!bounce || (remote_wins && ext) || sg > i))
            word = (uint32_t)inv[sg];
        else if (bounce)
            word = bounce_word(j, k, npad);
        else
            word = (uint32_t)n;
        nbr[(long long)(j - 1) * npad + k] = word;
    }
}

/* --------------------------------------------------------- state kernels */

template <typename T>
__device__ __forceinline__ void store_dev(T *p, float g);
template <> __device__ __forceinline__ void store_dev<float>(float *p, float g) { *p = g; }
template <> __device__ __forceinline__ void store_dev<__half>(__half *p, float g) { *p = __float2half_rn(g); }
template <> __device__ __forceinline__ void store_dev<__nv_bfloat16>(__nv_bfloat16 *p, float g) { *p = __float2bfloat16_rn(g); }
__device__ __forceinline__ double load_dev(const float *p) { return (double)*p; }
__device__ __forceinline__ double load_dev(const __half *p) { return (double)__half2float(*p); }
__device__ __forceinline__ double load_dev(const __nv_bfloat16 *p) { return (double)__bfloat162float(*p); }

__device__ __forceinline__ double wq(int j)
{
    return j == 0 ? 1.0 / 3 : (j <= 6 ? 1.0 / 18 : 1.0 / 36);
}

/* f = w (rest state) in all ping-pong buffers, rest slot included */
__global__ void k_init_fp64(double *f0, double *f1, long long npad, int n)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k > n) return;
#pragma unroll
    for (int j = 0; j < Q; j++) {
        f0[j * npad + k] = wq(j);
        f1[j * npad + k] = wq(j);
    }
}

template <typename T>
__global__ void k_init_dev(T *f0, T *f1, long long npad, int n)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k > n) return;
#pragma unroll
    for (int j = 0; j < Q; j++) {
        store_dev<T>(f0 + j * npad + k, 0.f);
        store_dev<T>(f1 + j * npad + k, 0.f);
    }
}

__global__ void k_init_macro(double *macro, long long npad, int n)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    macro[k] = 1.0;
    macro[npad + k] = 0.0;
    macro[2 * npad + k] = 0.0;
    macro[3 * npad + k] = 0.0;
}

__global__ void k_get_f_fp64(const double *f, const int *perm, long long npad,
                             int n, double *out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long o = (long long)perm[k] * Q;
#pragma unroll
    for (int j = 0; j < Q; j++) out[o + j] = f[j * npad + k];
}

template <typename T>
__global__ void k_get_f_dev(const T *f, const int *perm, long long npad, int n,
                            float inv_scale, double *out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long o = (long long)perm[k] * Q;
#pragma unroll
    for (int j = 0; j < Q; j++) {
        const double g = load_dev(f + j * npad + k) * (double)inv_scale;
        out[o + j] = wq(j) + wq(j) * g;
    }
}

/* the next step's streamed values (through the pull words), FP64 AoS */
template <typename T>
__global__ void k_get_streamed(const T *f, const uint32_t *nbr, const int *perm,
                               long long npad, int n, float inv_scale, double *out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long o = (long long)perm[k] * Q;
#pragma unroll
    for (int j = 0; j < Q; j++) {
        const long long at = j == 0 ? k : (long long)j * npad + (int)nbr[(j - 1) * npad + k];
        if constexpr (sizeof(T) == 8) {
            out[o + j] = ((const double *)f)[at];
        } else {
            const double g = load_dev(f + at) * (double)inv_scale;
            out[o + j] = wq(j) + wq(j) * g;
        }
    }
}

__global__ void k_set_f_fp64(double *f, const int *perm, long long npad, int n,
                             const double *in)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long o = (long long)perm[k] * Q;
#pragma unroll
    for (int j = 0; j < Q; j++) f[j * npad + k] = in[o + j];
}

template <typename T>
__global__ void k_set_f_dev(T *f, const int *perm, long long npad, int n,
                            float scale, const double *in)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long o = (long long)perm[k] * Q;
#pragma unroll
    for (int j = 0; j < Q; j++) {
        const double g = (in[o + j] - wq(j)) / wq(j);
        store_dev<T>(f + j * npad + k, (float)(g * (double)scale));
    }
}

__global__ void k_get_macro(const double *macro, const int *perm,
                            long long npad, int n, double *out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long o = perm[k];
#pragma unroll
    for (int c = 0; c < 4; c++) out[c * (long long)n + o] = macro[c * npad + k];
}

/* deterministic sum of the per-block partials: sums[0] = sum ux, [1] = rho */
__global__ void __launch_bounds__(1024)
k_sum_partials(const double *partial, int nb, double *sums)
{
    __shared__ double su[32], sr[32];
    double tu = 0.0, tr = 0.0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        tu += partial[k];
        tr += partial[nb + k];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tu += __shfl_down_sync(0xffffffffu, tu, o);
        tr += __shfl_down_sync(0xffffffffu, tr, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { su[wid] = tu; sr[wid] = tr; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) { a += su[k]; b += sr[k]; }
        sums[0] = a;
        sums[1] = b;
    }
}

/* ------------------------------------------------------------------ API */

static inline unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

static size_t elem_size(int precision)
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

static void free_sim(plb_sim *s)
{
    if (!s) return;
    cudaFree(s->f[0]);
    cudaFree(s->f[1]);
    cudaFree(s->nbr);
    cudaFree(s->perm);
    cudaFree(s->coord);
    cudaFree(s->macro);
    cudaFree(s->partial);
    cudaFree(s->sums);
    cudaFree(s->err);
    cudaFree(s->flags);
    if (s->stream) cudaStreamDestroy(s->stream);
    free(s->v_sub_start);
    free(s);
}

void plb_destroy(plb_sim *sim)
{
    if (!sim) return;
    cudaSetDevice(sim->device);
    cudaStreamSynchronize(sim->stream);
    free_sim(sim);
}

template <typename P>
static cudaError_t dev_alloc(P **p, size_t bytes, size_t *acc)
{
    *acc += bytes;
    return plb_cuda_malloc((void **)p, bytes ? bytes : 16);
}

static int build_tables(plb_sim *s, const plb_node_info *V_host)
{
    const int n = s->n;
    cudaStream_t st = s->stream;
    plb_node_info *dV = nullptr;
    int *inv = nullptr, *dstart = nullptr;
    unsigned *bad = nullptr;
    uint32_t *bitmap = nullptr, *cnt = nullptr, *offs = nullptr, *tmp = nullptr;
    int rc = PLB_OK;
    size_t scratch = 0;
#define CKT(call)                                                           \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                            \
            fprintf(stderr, "porelb_gpu: %s failed: %s\n", #call,           \
                    cudaGetErrorString(e_));                                \
            rc = (e_ == cudaErrorMemoryAllocation) ? PLB_ERR_NOMEM : PLB_ERR_CUDA; \
            goto done;                                                      \
        }                                                                   \
    } while (0)
    CKT(dev_alloc(&dV, sizeof(plb_node_info) * (size_t)n, &scratch));
    CKT(dev_alloc(&inv, sizeof(int) * (size_t)n, &scratch));
    CKT(dev_alloc(&dstart, sizeof(int) * (size_t)(s->num_p + 1), &scratch));
    CKT(dev_alloc(&bad, sizeof(unsigned), &scratch));
    CKT(cudaMemsetAsync(bad, 0, sizeof(unsigned), st));
    CKT(cudaMemcpyAsync(dV, V_host, sizeof(plb_node_info) * (size_t)n,
                        cudaMemcpyHostToDevice, st));
    CKT(cudaMemcpyAsync(dstart, s->v_sub_start, sizeof(int) * (size_t)(s->num_p + 1),
                        cudaMemcpyHostToDevice, st));
    CKT(cudaMemsetAsync(s->perm, 0xff, sizeof(int) * (size_t)s->npad, st));
    /* The Morton pass also validates the records (coordinates inside the
     * box, no two nodes on one cell: a repeated cell leaves a hole in the
     * numbering), so it runs for every order; in row order its numbering
     * is then replaced by the identity. */
    if (n > 0 && ceil_log2(s->nx) + ceil_log2(s->ny) + ceil_log2(s->nz) > 40 &&
        s->ordering == PLB_ORDER_REFERENCE) {
        k_identity<<<nblk(n, 256), 256, 0, st>>>(s->perm, inv, n);
    } else if (n > 0) {
        MortonBits b{ceil_log2(s->nx), ceil_log2(s->ny), ceil_log2(s->nz)};
        const int bits = b.bx + b.by + b.bz;
        if (bits > 40) {
            rc = PLB_ERR_ARG;
            goto done;
        }
        const size_t words = bits >= 5 ? ((size_t)1 << (bits - 5)) : 1;
        const size_t ntiles = (words + kScanTile - 1) / kScanTile;
        CKT(dev_alloc(&bitmap, words * 4, &scratch));
        CKT(dev_alloc(&cnt, words * 4, &scratch));
        CKT(dev_alloc(&offs, words * 4, &scratch));
        CKT(dev_alloc(&tmp, ntiles * 4 + 4, &scratch));
        CKT(cudaMemsetAsync(bitmap, 0, words * 4, st));
        k_morton_mark<<<nblk(n, 256), 256, 0, st>>>(dV, n, s->nx, s->ny, s->nz, b, bitmap, bad);
        k_popc<<<nblk((long long)words, 256), 256, 0, st>>>(bitmap, cnt, words);
        CKT(cudaGetLastError());
        rc = exclusive_scan(cnt, offs, words, tmp, st);
        if (rc != PLB_OK) goto done;
        k_morton_assign<<<nblk(n, 256), 256, 0, st>>>(dV, n, s->nx, s->ny, s->nz, b, bitmap,
                                                     offs, s->perm, inv, bad);
        if (s->ordering != PLB_ORDER_MORTON) {
            k_perm_holes<<<nblk(n, 256), 256, 0, st>>>(s->perm, n, bad);
            k_identity<<<nblk(n, 256), 256, 0, st>>>(s->perm, inv, n);
        }
    }
    CKT(cudaGetLastError());
    if (n > 0) {
        const int remote_wins = (s->halo == PLB_HALO_REMOTE_WINS) ||
                                (s->halo == PLB_HALO_AUTO && s->num_p > 1);
        k_build_nbr<<<nblk(n, 128), 128, 0, st>>>(dV, s->perm, inv, dstart, s->num_p, n,
                                                 s->npad, remote_wins, s->boundary,
                                                 s->nbr, s->coord, bad);
        CKT(cudaGetLastError());
    }
    {
        unsigned hbad = 0;
        CKT(cudaMemcpyAsync(&hbad, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        CKT(cudaStreamSynchronize(st));
        if (hbad) {
            fprintf(stderr, "porelb_gpu: node table rejected (flags 0x%x)\n", hbad);
            rc = PLB_ERR_TABLE;
        }
    }
done:
    cudaStreamSynchronize(st);
    cudaFree(dV);
    cudaFree(inv);
    cudaFree(dstart);
    cudaFree(bad);
    cudaFree(bitmap);
    cudaFree(cnt);
    cudaFree(offs);
    cudaFree(tmp);
#undef CKT
    return rc;
}

/* Validate the parameters, create the handle and allocate its device arrays
 * for n nodes (everything but the tables). */
static int sim_alloc(const plb_params *p, int n, int nx, int ny, int nz,
                     int num_p, const int *v_sub_start, plb_sim **out)
{
    *out = nullptr;
    if (n < 0 || nx <= 0 || ny <= 0 || nz <= 0 || num_p <= 0 || !v_sub_start ||
        !(p->tau > 0.5) || !isfinite(p->force_x) || elem_size(p->precision) == 0 ||
        (p->ordering != PLB_ORDER_MORTON && p->ordering != PLB_ORDER_REFERENCE &&
         p->ordering != PLB_ORDER_AUTO) ||
        (p->boundary != PLB_BOUNDARY_REFERENCE && p->boundary != PLB_BOUNDARY_HALFWAY) ||
        n >= kMaxNodes)
        return PLB_ERR_ARG;
    if (v_sub_start[0] != 0) return PLB_ERR_NUMP;
    for (int q = 0; q < num_p; q++) {
        const int hi = q + 1 < num_p ? v_sub_start[q + 1] : n;
        if (v_sub_start[q] < 0 || hi < v_sub_start[q] || hi > n) return PLB_ERR_NUMP;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0 || p->device < 0 ||
        p->device >= ndev) {
        fprintf(stderr, "porelb_gpu: no usable CUDA device\n");
        return PLB_ERR_CUDA;
    }
    CK(cudaSetDevice(p->device));
    plb_sim *s = (plb_sim *)calloc(1, sizeof(plb_sim));
    if (!s) return PLB_ERR_NOMEM;
    s->n = n;
    s->nx = nx; s->ny = ny; s->nz = nz;
    s->num_p = num_p;
    s->npad = ((long long)n + 1 + 63) / 64 * 64;
    s->precision = p->precision;
    s->ordering = p->ordering == PLB_ORDER_AUTO
                      ? plb_auto_ordering(n, nz, (int)elem_size(p->precision), p->device)
                      : p->ordering;
    s->halo = p->halo;
    s->boundary = p->boundary;
    /* register budget of the step kernel (kernel_variant 1 and 3 are the
     * alternatives; for FP64 the default 128-register kernel is the faster on
     * GB300 - every tighter budget spills: 96 to 120 registers ran at 13.5 to
     * 15.2 GLUPS at 256^3 against 16.2) */
    s->variant = p->kernel_variant == 1 ? 1 : (p->kernel_variant == 3 ? 3 : 0);
    s->block = p->block_size > 0 ? p->block_size
                                 : (p->precision == PLB_FP64 ? 128 : 256);
    if (s->block > 256 || (s->block & 31)) s->block = 256;
    /* prefetching the next wave into L2 pays for the issue-bound FP64 form
     * (+5% at 256^3 and 512^3) and costs the bandwidth-bound forms (FP32
     * -13%, FP16 deviations up to -11%) */
    s->prefetch = p->l2_prefetch > 0 || (p->l2_prefetch == 0 && p->precision == PLB_FP64);
    s->device = p->device;
    s->elem = elem_size(p->precision);
    s->tau = p->tau;
    s->force = p->force_x;
    plb_host_constants(p->tau, p->force_x, &s->omega, &s->om1, &s->k3,
                       &s->half_force, &s->nu);
    s->fxk = fx::make_consts(p->tau, p->force_x);
    s->scale = p->precision == PLB_FP16DEV ? 1024.0f : 1.0f;
    s->v_sub_start = (int *)malloc(sizeof(int) * (size_t)(num_p + 1));
    if (!s->v_sub_start) { free(s); return PLB_ERR_NOMEM; }
    memcpy(s->v_sub_start, v_sub_start, sizeof(int) * (size_t)num_p);
    s->v_sub_start[num_p] = n;
    s->nblocks = (int)nblk(n > 0 ? n : 1, s->block);

    size_t acc = 0;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    const size_t fbytes = s->elem * Q * (size_t)s->npad;
    if (e == cudaSuccess) e = dev_alloc(&s->f[0], fbytes, &acc);
    if (e == cudaSuccess) e = dev_alloc(&s->f[1], fbytes, &acc);
    if (e == cudaSuccess) e = dev_alloc(&s->nbr, 4 * 18 * (size_t)s->npad, &acc);
    if (e == cudaSuccess) e = dev_alloc(&s->perm, 4 * (size_t)s->npad, &acc);
    if (e == cudaSuccess) e = dev_alloc(&s->coord, 2 * 3 * (size_t)s->npad, &acc);
    if (e == cudaSuccess) e = dev_alloc(&s->macro, 8 * 4 * (size_t)s->npad, &acc);
    if (e == cudaSuccess) e = dev_alloc(&s->partial, 8 * 2 * (size_t)s->nblocks, &acc);
    if (e == cudaSuccess) e = dev_alloc(&s->sums, 16, &acc);
    if (e == cudaSuccess) e = dev_alloc(&s->err, 8, &acc);
    if (e == cudaSuccess) e = dev_alloc(&s->flags, 4, &acc);
    if (e != cudaSuccess) {
        fprintf(stderr, "porelb_gpu: allocation failed: %s\n", cudaGetErrorString(e));
        free_sim(s);
        return e == cudaErrorMemoryAllocation ? PLB_ERR_NOMEM : PLB_ERR_CUDA;
    }
    s->dev_bytes = acc;
    *out = s;
    return PLB_OK;
}

static int sim_finish(plb_sim *s, int rc, plb_sim **out)
{
    if (rc == PLB_OK) {
        cudaError_t e = cudaMemsetAsync(s->err, 0xff, 8, s->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->flags, 0, 4, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) rc = PLB_ERR_CUDA;
    }
    if (rc != PLB_OK) {
        free_sim(s);
        *out = nullptr;
        return rc;
    }
    *out = s;
    return PLB_OK;
}

int plb_create(const plb_node_info *V, int num_node, int nx, int ny, int nz,
               int num_p, const int *v_sub_start, const plb_params *p,
               plb_sim **out)
{
    if (!out) return PLB_ERR_ARG;
    *out = nullptr;
    plb_params defp;
    if (!p) {
        plb_default_params(&defp);
        p = &defp;
    }
    if (num_node < 0 || (num_node > 0 && !V)) return PLB_ERR_ARG;
    plb_sim *s = nullptr;
    int rc = sim_alloc(p, num_node, nx, ny, nz, num_p, v_sub_start, &s);
    if (rc != PLB_OK) return rc;
    return sim_finish(s, build_tables(s, V), out);
}

/* Tables from a flag grid already on the device. */
static int create_from_dflag(const uint8_t *dflag, int nx, int ny, int nz,
                             int num_p, const plb_params *p, cudaStream_t st,
                             plb_sim **out)
{
    const size_t cells = (size_t)nx * ny * nz;
    const size_t words = (cells + 31) / 32;
    uint32_t *lexbits = nullptr, *lexoffs = nullptr;
    int *slab = (int *)calloc((size_t)num_p + 1, sizeof(int));
    int rc = PLB_OK, n = 0;
    plb_sim *s = nullptr;
    if (!slab) return PLB_ERR_NOMEM;
    if (plb_cuda_malloc(&lexbits, words * 4) != cudaSuccess ||
        plb_cuda_malloc(&lexoffs, words * 4) != cudaSuccess) {
        rc = PLB_ERR_NOMEM;
    }
    if (rc == PLB_OK)
        rc = flag_rank(dflag, nx, ny, nz, num_p, lexbits, lexoffs, &n, slab, st);
    if (rc == PLB_OK) rc = sim_alloc(p, n, nx, ny, nz, num_p, slab, &s);
    if (rc == PLB_OK) {
        const int remote_wins = (s->halo == PLB_HALO_REMOTE_WINS) ||
                                (s->halo == PLB_HALO_AUTO && s->num_p > 1);
        rc = flag_tables(dflag, nx, ny, nz, num_p, s->ordering, remote_wins,
                         s->boundary, lexbits, lexoffs, n, s->npad, s->perm, s->coord,
                         s->nbr, 0u, (uint32_t)n, st);
        rc = sim_finish(s, rc, out);
    }
    cudaFree(lexbits);
    cudaFree(lexoffs);
    free(slab);
    return rc;
}

int plb_create_from_flag(const uint8_t *flag, int nx, int ny, int nz,
                         int num_p, const plb_params *p, plb_sim **out)
{
    if (!out) return PLB_ERR_ARG;
    *out = nullptr;
    plb_params defp;
    if (!p) {
        plb_default_params(&defp);
        p = &defp;
    }
    if (!flag || nx <= 0 || ny <= 0 || nz <= 0 || nx > 65536 || ny > 65536 ||
        nz > 65536 || num_p <= 0 || num_p > nz || nz % num_p)
        return PLB_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0 || p->device < 0 ||
        p->device >= ndev)
        return PLB_ERR_CUDA;
    CK(cudaSetDevice(p->device));
    const size_t cells = (size_t)nx * ny * nz;
    uint8_t *dflag = nullptr;
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int rc = PLB_OK;
    if (plb_cuda_malloc(&dflag, cells) != cudaSuccess) rc = PLB_ERR_NOMEM;
    if (rc == PLB_OK && cudaMemcpyAsync(dflag, flag, cells, cudaMemcpyHostToDevice, st) != cudaSuccess)
        rc = PLB_ERR_CUDA;
    if (rc == PLB_OK) rc = create_from_dflag(dflag, nx, ny, nz, num_p, p, st, out);
    cudaStreamSynchronize(st);
    cudaFree(dflag);
    cudaStreamDestroy(st);
    return rc;
}

int plb_sphere_pack_device(uint64_t seed, int nx, int ny, int nz, double rmin,
                           double rmax, double porosity, int device,
                           uint8_t *flag, int *num_spheres, double *porosity_out)
{
    if (nx <= 0 || ny <= 0 || nz <= 0 || !(rmin > 0.0) || rmax < rmin ||
        !(porosity >= 0.0) || !(porosity <= 1.0))
        return PLB_ERR_ARG;
    CK(cudaSetDevice(device));
    const size_t cells = (size_t)nx * ny * nz;
    uint8_t *dflag = nullptr;
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int rc = PLB_OK;
    if (plb_cuda_malloc(&dflag, cells) != cudaSuccess) rc = PLB_ERR_NOMEM;
    if (rc == PLB_OK)
        rc = sphere_pack_device(seed, nx, ny, nz, rmin, rmax, porosity, dflag,
                                num_spheres, porosity_out, st);
    if (rc == PLB_OK && flag &&
        (cudaMemcpyAsync(flag, dflag, cells, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
         cudaStreamSynchronize(st) != cudaSuccess))
        rc = PLB_ERR_CUDA;
    cudaStreamSynchronize(st);
    cudaFree(dflag);
    cudaStreamDestroy(st);
    return rc;
}

int plb_create_packed(uint64_t seed, int nx, int ny, int nz, double rmin,
                      double rmax, double porosity, int num_p,
                      const plb_params *p, plb_sim **out, int *num_spheres,
                      double *porosity_out)
{
    if (!out) return PLB_ERR_ARG;
    *out = nullptr;
    plb_params defp;
    if (!p) {
        plb_default_params(&defp);
        p = &defp;
    }
    if (nx <= 0 || ny <= 0 || nz <= 0 || nx > 65536 || ny > 65536 || nz > 65536 ||
        num_p <= 0 || num_p > nz || nz % num_p || !(rmin > 0.0) || rmax < rmin ||
        !(porosity >= 0.0) || !(porosity <= 1.0))
        return PLB_ERR_ARG;
    CK(cudaSetDevice(p->device));
    const size_t cells = (size_t)nx * ny * nz;
    uint8_t *dflag = nullptr;
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int rc = PLB_OK;
    if (plb_cuda_malloc(&dflag, cells) != cudaSuccess) rc = PLB_ERR_NOMEM;
    if (rc == PLB_OK)
        rc = sphere_pack_device(seed, nx, ny, nz, rmin, rmax, porosity, dflag,
                                num_spheres, porosity_out, st);
    if (rc == PLB_OK) rc = create_from_dflag(dflag, nx, ny, nz, num_p, p, st, out);
    cudaStreamSynchronize(st);
    cudaFree(dflag);
    cudaStreamDestroy(st);
    return rc;
}

int plb_init_equilibrium(plb_sim *s)
{
    if (!s) return PLB_ERR_ARG;
    CK(cudaSetDevice(s->device));
    const unsigned g = nblk(s->npad, 256);
    switch (s->precision) {
    case PLB_FP64_EXACT:
    case PLB_FP64:
    case PLB_FP64_FMA:
        k_init_fp64<<<g, 256, 0, s->stream>>>((double *)s->f[0], (double *)s->f[1], s->npad, s->n);
        break;
    case PLB_FP32:
        k_init_dev<float><<<g, 256, 0, s->stream>>>((float *)s->f[0], (float *)s->f[1], s->npad, s->n);
        break;
    case PLB_FP16DEV:
        k_init_dev<__half><<<g, 256, 0, s->stream>>>((__half *)s->f[0], (__half *)s->f[1], s->npad, s->n);
        break;
    default:
        k_init_dev<__nv_bfloat16><<<g, 256, 0, s->stream>>>((__nv_bfloat16 *)s->f[0],
                                                           (__nv_bfloat16 *)s->f[1], s->npad, s->n);
        break;
    }
    if (s->n > 0) k_init_macro<<<nblk(s->n, 256), 256, 0, s->stream>>>(s->macro, s->npad, s->n);
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(s->err, 0xff, 8, s->stream));
    CK(cudaMemsetAsync(s->flags, 0, 4, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    s->cur = 0;
    s->initialized = 1;
    s->fallback_nodes_seen = 0;
    s->macro_valid = 1;
    s->err_it = -1;
    s->err_node = -1;
    return PLB_OK;
}

int plb_step_async(plb_sim *s, int it_begin, int nsteps)
{
    if (!s || nsteps < 0 || it_begin < 0) return PLB_ERR_ARG;
    if (!s->initialized) return PLB_ERR_STATE;
    if (nsteps == 0) return PLB_OK;
    CK(cudaSetDevice(s->device));
    StepArgs a;
    memset(&a, 0, sizeof(a));
    a.nbr = s->nbr;
    a.perm = s->perm;
    a.npad = s->npad;
    a.n = s->n;
    make_coeffs(s->tau, s->force, s->scale, &a.co);
    a.macro = s->macro;
    a.partial = s->partial;
    a.err = s->err;
    a.flags = s->flags;
    if (s->prefetch && s->wave == 0) s->wave = step_wave_blocks(s->precision, s->block, s->variant);
    /* half a wave of resident blocks ahead (measured at 256^3 and 512^3:
     * +0.7% against a whole wave, +7% against no prefetch) */
    a.pf_blocks = s->prefetch ? (s->wave + 1) / 2 : 0;
    for (int k = 0; k < nsteps; k++) {
        a.fin = s->f[s->cur];
        a.fout = s->f[s->cur ^ 1];
        a.co.it = it_begin + k;
        const bool last = (k == nsteps - 1);
        cudaError_t e = launch_step(s->precision, last, a, s->block, s->variant, s->stream);
        if (e != cudaSuccess) {
            fprintf(stderr, "porelb_gpu: step launch failed: %s\n", cudaGetErrorString(e));
            return PLB_ERR_CUDA;
        }
        s->cur ^= 1;
    }
    s->macro_valid = 1;
    return PLB_OK;
}

int plb_sync(plb_sim *s)
{
    if (!s) return PLB_ERR_ARG;
    CK(cudaSetDevice(s->device));
    unsigned long long key = ~0ull;
    unsigned flags = 0;
    CK(cudaMemcpyAsync(&key, s->err, 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(&flags, s->flags, 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (key != ~0ull) {
        s->err_it = (int)(key >> 32);
        s->err_node = (int)(key & 0xffffffffu);
        return PLB_ERR_DENSITY;
    }
    if (flags & 2u) s->fallback_nodes_seen = 1;
    if (flags & 1u) {
        fprintf(stderr, "porelb_gpu: FP16 deviation overflow; lower the scale\n");
        return PLB_ERR_STATE;
    }
    return PLB_OK;
}

int plb_step(plb_sim *s, int it_begin, int nsteps)
{
    int rc = plb_step_async(s, it_begin, nsteps);
    if (rc != PLB_OK) return rc;
    return plb_sync(s);
}

int plb_get_macros(plb_sim *s, double *rho, double *ux, double *uy, double *uz)
{
    if (!s) return PLB_ERR_ARG;
    if (!s->macro_valid) return PLB_ERR_STATE;
    if (s->n == 0) return PLB_OK;
    CK(cudaSetDevice(s->device));
    double *d = nullptr;
    CK(plb_cuda_malloc(&d, sizeof(double) * 4 * (size_t)s->n));
    k_get_macro<<<nblk(s->n, 256), 256, 0, s->stream>>>(s->macro, s->perm, s->npad, s->n, d);
    double *dst[4] = {rho, ux, uy, uz};
    cudaError_t e = cudaGetLastError();
    for (int c = 0; c < 4 && e == cudaSuccess; c++)
        if (dst[c])
            e = cudaMemcpyAsync(dst[c], d + (size_t)c * s->n, sizeof(double) * (size_t)s->n,
                                cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) {
        fprintf(stderr, "porelb_gpu: get_macros failed: %s\n", cudaGetErrorString(e));
        return PLB_ERR_CUDA;
    }
    return PLB_OK;
}

int plb_save_parts(plb_sim *s, const char *dir, int tag)
{
    if (!s) return PLB_ERR_ARG;
    double *buf = (double *)malloc(sizeof(double) * 4 * (size_t)(s->n ? s->n : 1));
    if (!buf) return PLB_ERR_NOMEM;
    const size_t n = (size_t)s->n;
    int rc = plb_get_macros(s, buf, buf + n, buf + 2 * n, buf + 3 * n);
    for (int p = 0; p < s->num_p && rc == PLB_OK; p++) {
        char name[4096];
        snprintf(name, sizeof(name), "%s%spart_%03d_%07d.bin", dir ? dir : "",
                 (dir && dir[0] && dir[strlen(dir) - 1] != '/') ? "/" : "", p, tag);
        FILE *fp = fopen(name, "wb");
        if (!fp) { rc = PLB_ERR_IO; break; }
        const size_t lo = (size_t)s->v_sub_start[p], cnt = (size_t)s->v_sub_start[p + 1] - lo;
        for (int c = 0; c < 4; c++)
            if (fwrite(buf + c * n + lo, sizeof(double), cnt, fp) != cnt) rc = PLB_ERR_IO;
        if (fclose(fp) != 0) rc = PLB_ERR_IO;
    }
    free(buf);
    return rc;
}

int plb_get_f(plb_sim *s, double *f_aos)
{
    if (!s || (!f_aos && s->n > 0)) return PLB_ERR_ARG;
    if (!s->initialized) return PLB_ERR_STATE;
    if (s->n == 0) return PLB_OK;
    CK(cudaSetDevice(s->device));
    double *d = nullptr;
    const size_t bytes = sizeof(double) * Q * (size_t)s->n;
    CK(plb_cuda_malloc(&d, bytes));
    const unsigned g = nblk(s->n, 256);
    const void *f = s->f[s->cur];
    switch (s->precision) {
    case PLB_FP64_EXACT:
    case PLB_FP64:
    case PLB_FP64_FMA: k_get_f_fp64<<<g, 256, 0, s->stream>>>((const double *)f, s->perm, s->npad, s->n, d); break;
    case PLB_FP32: k_get_f_dev<float><<<g, 256, 0, s->stream>>>((const float *)f, s->perm, s->npad, s->n, 1.0f / s->scale, d); break;
    case PLB_FP16DEV: k_get_f_dev<__half><<<g, 256, 0, s->stream>>>((const __half *)f, s->perm, s->npad, s->n, 1.0f / s->scale, d); break;
    default: k_get_f_dev<__nv_bfloat16><<<g, 256, 0, s->stream>>>((const __nv_bfloat16 *)f, s->perm, s->npad, s->n, 1.0f / s->scale, d); break;
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(f_aos, d, bytes, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) {
        fprintf(stderr, "porelb_gpu: get_f failed: %s\n", cudaGetErrorString(e));
        return PLB_ERR_CUDA;
    }
    return PLB_OK;
}

int plb_set_f(plb_sim *s, const double *f_aos)
{
    if (!s || (!f_aos && s->n > 0)) return PLB_ERR_ARG;
    if (!s->initialized) return PLB_ERR_STATE;
    if (s->n == 0) return PLB_OK;
    CK(cudaSetDevice(s->device));
    double *d = nullptr;
    const size_t bytes = sizeof(double) * Q * (size_t)s->n;
    CK(plb_cuda_malloc(&d, bytes));
    cudaError_t e = cudaMemcpyAsync(d, f_aos, bytes, cudaMemcpyHostToDevice, s->stream);
    const unsigned g = nblk(s->n, 256);
    void *f = s->f[s->cur];
    if (e == cudaSuccess) {
        switch (s->precision) {
        case PLB_FP64_EXACT:
        case PLB_FP64:
        case PLB_FP64_FMA: k_set_f_fp64<<<g, 256, 0, s->stream>>>((double *)f, s->perm, s->npad, s->n, d); break;
        case PLB_FP32: k_set_f_dev<float><<<g, 256, 0, s->stream>>>((float *)f, s->perm, s->npad, s->n, s->scale, d); break;
        case PLB_FP16DEV: k_set_f_dev<__half><<<g, 256, 0, s->stream>>>((__half *)f, s->perm, s->npad, s->n, s->scale, d); break;
        default: k_set_f_dev<__nv_bfloat16><<<g, 256, 0, s->stream>>>((__nv_bfloat16 *)f, s->perm, s->npad, s->n, s->scale, d); break;
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) {
        fprintf(stderr, "porelb_gpu: set_f failed: %s\n", cudaGetErrorString(e));
        return PLB_ERR_CUDA;
    }
    return PLB_OK;
}

int plb_get_f_streamed(plb_sim *s, double *f_aos)
{
    if (!s || (!f_aos && s->n > 0)) return PLB_ERR_ARG;
    if (!s->initialized) return PLB_ERR_STATE;
    if (s->n == 0) return PLB_OK;
    CK(cudaSetDevice(s->device));
    double *d = nullptr;
    const size_t bytes = sizeof(double) * Q * (size_t)s->n;
    CK(plb_cuda_malloc(&d, bytes));
    const unsigned g = nblk(s->n, 256);
    const void *f = s->f[s->cur];
    const float inv = 1.0f / s->scale;
    switch (s->precision) {
    case PLB_FP64_EXACT:
    case PLB_FP64:
    case PLB_FP64_FMA: k_get_streamed<double><<<g, 256, 0, s->stream>>>((const double *)f, s->nbr, s->perm, s->npad, s->n, inv, d); break;
    case PLB_FP32: k_get_streamed<float><<<g, 256, 0, s->stream>>>((const float *)f, s->nbr, s->perm, s->npad, s->n, inv, d); break;
    case PLB_FP16DEV: k_get_streamed<__half><<<g, 256, 0, s->stream>>>((const __half *)f, s->nbr, s->perm, s->npad, s->n, inv, d); break;
    default: k_get_streamed<__nv_bfloat16><<<g, 256, 0, s->stream>>>((const __nv_bfloat16 *)f, s->nbr, s->perm, s->npad, s->n, inv, d); break;
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(f_aos, d, bytes, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) {
        fprintf(stderr, "porelb_gpu: get_f_streamed failed: %s\n", cudaGetErrorString(e));
        return PLB_ERR_CUDA;
    }
    return PLB_OK;
}

int plb_reduce(plb_sim *s, double *sum_ux, double *mass)
{
    if (!s) return PLB_ERR_ARG;
    if (!s->macro_valid) return PLB_ERR_STATE;
    CK(cudaSetDevice(s->device));
    double h[2] = {0.0, 0.0};
    if (s->n > 0) {
        if (!s->initialized) return PLB_ERR_STATE;
        k_sum_partials<<<1, 1024, 0, s->stream>>>(s->partial, s->nblocks, s->sums);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(h, s->sums, 16, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    if (sum_ux) *sum_ux = h[0];
    if (mass) *mass = h[1];
    return PLB_OK;
}

int plb_permeability(plb_sim *s, double *k_darcy, double *k_intrinsic)
{
    double su = 0.0;
    int rc = plb_reduce(s, &su, nullptr);
    if (rc != PLB_OK) return rc;
    if (s->force == 0.0) return PLB_ERR_ARG;
    const double cells = (double)s->nx * s->ny * s->nz;
    if (k_darcy) *k_darcy = su / cells * s->nu / s->force;
    if (k_intrinsic) *k_intrinsic = s->n ? su / s->n * s->nu / s->force : 0.0;
    return PLB_OK;
}

int plb_last_error(plb_sim *s, int *it, int *node, int *x, int *y, int *z,
                   double *rho)
{
    if (!s) return PLB_ERR_ARG;
    if (s->err_node < 0) return PLB_OK;
    if (it) *it = s->err_it;
    if (node) *node = s->err_node;
    if (rho) *rho = NAN;
    if (x || y || z) {
        /* coordinates of the reported node: find its position in new order */
        int k = -1;
        int *hp = (int *)malloc(sizeof(int) * (size_t)s->n);
        if (hp && cudaMemcpy(hp, s->perm, sizeof(int) * (size_t)s->n,
                             cudaMemcpyDeviceToHost) == cudaSuccess)
            for (int q = 0; q < s->n; q++)
                if (hp[q] == s->err_node) { k = q; break; }
        free(hp);
        uint16_t c[3] = {0, 0, 0};
        if (k >= 0)
            for (int d = 0; d < 3; d++)
                cudaMemcpy(&c[d], s->coord + (size_t)d * s->npad + k, 2, cudaMemcpyDeviceToHost);
        if (x) *x = c[0];
        if (y) *y = c[1];
        if (z) *z = c[2];
    }
    return PLB_ERR_DENSITY;
}

int plb_kernel_flags(plb_sim *s, unsigned *flags)
{
    if (!s || !flags) return PLB_ERR_ARG;
    *flags = s->fallback_nodes_seen ? PLB_FLAG_FX_FALLBACK : 0u;
    return PLB_OK;
}

int plb_info(plb_sim *s, int *num_node, int *npad, int *precision,
             size_t *device_bytes)
{
    if (!s) return PLB_ERR_ARG;
    if (num_node) *num_node = s->n;
    if (npad) *npad = (int)s->npad;
    if (precision) *precision = s->precision;
    if (device_bytes) *device_bytes = s->dev_bytes;
    return PLB_OK;
}

void *plb_stream(plb_sim *s) { return s ? (void *)s->stream : nullptr; }
