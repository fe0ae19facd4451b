/*
 * plb_noalloc.cu - the macro reduction (sum of Ux and of Rho) without any
 * device allocation.
 *
 * plb_reduce sums the per-block partials that the solver's last step wrote
 * into memory its handle allocated.  Some callers cannot let a library
 * allocate device memory: a host framework that owns all device memory
 * through its own pool and budget (a stray cudaMalloc escapes its accounting
 * and can fail under its cap), a serving loop admitting work against a fixed
 * HBM budget, or code that must not synchronise the device (cudaMalloc and
 * cudaFree can).  plb_reduce_noalloc takes the caller's device arrays and
 * output and keeps its per-block partials in one file-scope device array of
 * fixed size, which exists on every GPU that loads this library until the
 * process exits.
 *
 * Every call shares that array: it keeps the last call's partials, each
 * call overwrites the slots it reads before reading them (nothing needs to
 * start at zero), and calls that overlap on the GPU - on different streams
 * of the same device - race on it.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress); make that first call before
 * any stream capture.
 */
#include <stdio.h>

#include <mutex>

#include "plb_internal.h"

namespace {

constexpr int kThreads = 256;
/* per-block partial pairs: at most this many 256-node blocks per call */
constexpr long long kMaxBlocks = 1LL << 18;
static_assert(kMaxBlocks * kThreads == PLB_REDUCE_NOALLOC_MAX_NODES,
              "header limit and scratch size disagree");

/* 2 * 2^18 doubles = 4 MiB on every device that loads the library */
static __device__ __align__(256) double g_partials[2 * kMaxBlocks];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_partials_addr[kMaxDevices] = {nullptr};

__global__ void k_partials(const double *ux, const double *rho, long long n,
                           double *part)
{
    __shared__ double su[kThreads / 32], sr[kThreads / 32];
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    double a = 0.0, r = 0.0;
    if (i < n) {
        a = ux[i];
        r = rho[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        r += __shfl_down_sync(0xffffffffu, r, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { su[wid] = a; sr[wid] = r; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tr = 0.0;
        for (int k = 0; k < kThreads / 32; k++) { ta += su[k]; tr += sr[k]; }
        part[blockIdx.x] = ta;
        part[kMaxBlocks + blockIdx.x] = tr;
    }
}

/* fixed-order sum of nb partial pairs -> out[0], out[1] */
__global__ void k_final(const double *part, long long nb, double *out)
{
    __shared__ double su[32], sr[32];
    double a = 0.0, r = 0.0;
    for (long long k = threadIdx.x; k < nb; k += blockDim.x) {
        a += part[k];
        r += part[kMaxBlocks + k];
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        r += __shfl_down_sync(0xffffffffu, r, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { su[wid] = a; sr[wid] = r; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tr = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) { ta += su[k]; tr += sr[k]; }
        out[0] = ta;
        out[1] = tr;
    }
}

}  // namespace

/* The device address of g_partials on the current device.  In host code
 * g_partials names a host-side stand-in, not device memory, so the address
 * is looked up once per device with that device current and kept.  The
 * cache is keyed by device ordinal and assumes the device's primary context
 * outlives the library's use: a context reset (cudaDeviceReset) may reload
 * the module at another address, which this cache would not see. */
static int partials_on_current_device(double **addr)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return PLB_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_partials_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_partials);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "porelb_gpu: cudaGetSymbolAddress failed: %s\n",
                    cudaGetErrorString(e));
            return PLB_ERR_CUDA;
        }
        g_partials_addr[dev] = (double *)p;
    }
    *addr = g_partials_addr[dev];
    return PLB_OK;
}

extern "C" int plb_reduce_noalloc(const double *ux, const double *rho,
                                  long long n, double *out, void *stream)
{
    if (n < 0 || !out || (n > 0 && (!ux || !rho))) return PLB_ERR_ARG;
    if (n > kMaxBlocks * kThreads) {
        fprintf(stderr, "porelb_gpu: plb_reduce_noalloc: %lld nodes exceed the "
                        "fixed scratch limit of %lld nodes\n",
                n, kMaxBlocks * kThreads);
        return PLB_ERR_ARG;
    }
    double *part = nullptr;
    int rc = partials_on_current_device(&part);
    if (rc != PLB_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const long long nb = (n + kThreads - 1) / kThreads;
    if (nb > 0) k_partials<<<(unsigned)nb, kThreads, 0, st>>>(ux, rho, n, part);
    k_final<<<1, 1024, 0, st>>>(part, nb, out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "porelb_gpu: plb_reduce_noalloc launch failed: %s\n",
                cudaGetErrorString(e));
        return PLB_ERR_CUDA;
    }
    return PLB_OK;
}
