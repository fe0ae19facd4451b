/*
 * plb_geom.cu - device-side geometry: the periodic sphere-pack generator and
 * the node table built straight from a flag grid.
 *
 * build_V (preprocess.c:29-164) numbers fluid cells (flag == 1) in x-fastest
 * lexicographic order and stores, per node, the 18 neighbours at x + e_j.
 * From a flag grid the same information is a bit test: here the fluid cells
 * are ranked twice with popcount scans over bitmaps - once in lexicographic
 * order (the reference node number, used for the dump order and for the
 * order-dependent bounce-back rule) and once along the Morton curve (the
 * device order) - and the pull table is written directly, without the
 * 152-byte-per-node V.bin records.  For a flag with values 0/1 the result is
 * identical to plb_create on the table plb_build_table writes.
 */
#include <stdio.h>

#include "plb_internal.h"

namespace plb {

/* ------------------------------------------------------------- bitmaps */

/* lexicographic fluid bitmap: word w covers cells 32w .. 32w+31 */
__global__ void k_flag_bits(const uint8_t *flag, size_t cells, uint32_t *bits,
                            uint32_t *cnt, size_t words, unsigned *bad)
{
    const size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= words) return;
    uint32_t b = 0;
    const size_t c0 = w * 32;
    for (int k = 0; k < 32; k++) {
        const size_t c = c0 + k;
        if (c < cells) {
            const uint8_t v = flag[c];
            if (v > 1) atomicOr(bad, 1u);
            b |= (uint32_t)(v == 1) << k;
        }
    }
    bits[w] = b;
    cnt[w] = __popc(b);
}

__device__ __forceinline__ uint32_t rank_in(const uint32_t *bits,
                                            const uint32_t *offs, uint64_t c)
{
    const uint32_t w = bits[c >> 5];
    return offs[c >> 5] + __popc(w & ((1u << (c & 31)) - 1u));
}

__device__ __forceinline__ bool bit_at(const uint32_t *bits, uint64_t c)
{
    return (bits[c >> 5] >> (c & 31)) & 1u;
}

__host__ __device__ inline uint64_t morton_code(uint32_t x, uint32_t y,
                                                uint32_t z, int bx, int by,
                                                int bz)
{
    uint64_t c = 0;
    int pos = 0;
    const int top = bx > by ? (bx > bz ? bx : bz) : (by > bz ? by : bz);
    for (int k = 0; k < top; k++) {
        if (k < bx) c |= (uint64_t)((x >> k) & 1u) << pos++;
        if (k < by) c |= (uint64_t)((y >> k) & 1u) << pos++;
        if (k < bz) c |= (uint64_t)((z >> k) & 1u) << pos++;
    }
    return c;
}

struct Grid {
    int nx, ny, nz;
    int bx, by, bz;
    int morton; /* 0 = device order is the reference order */
};

__device__ __forceinline__ uint64_t device_key(const Grid &g, int x, int y, int z)
{
    return g.morton ? morton_code(x, y, z, g.bx, g.by, g.bz)
                    : ((uint64_t)z * g.ny + y) * g.nx + x;
}

__global__ void k_mark_order(const uint32_t *lexbits, Grid g, size_t cells,
                             uint32_t *obits)
{
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells || !bit_at(lexbits, c)) return;
    const int x = (int)(c % g.nx);
    const int y = (int)((c / g.nx) % g.ny);
    const int z = (int)(c / ((size_t)g.nx * g.ny));
    const uint64_t k = device_key(g, x, y, z);
    atomicOr(obits + (k >> 5), 1u << (k & 31));
}

/* device index, reference index and coordinates of every fluid cell */
__global__ void k_assign_from_flag(const uint32_t *lexbits, const uint32_t *lexoffs,
                                   const uint32_t *obits, const uint32_t *ooffs,
                                   Grid g, size_t cells, int n, long long npad,
                                   int *perm, uint16_t *coord)
{
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells || !bit_at(lexbits, c)) return;
    const int x = (int)(c % g.nx);
    const int y = (int)((c / g.nx) % g.ny);
    const int z = (int)(c / ((size_t)g.nx * g.ny));
    const uint32_t k = rank_in(obits, ooffs, device_key(g, x, y, z));
    if (k >= (uint32_t)n) return;
    perm[k] = (int)rank_in(lexbits, lexoffs, c);
    coord[k] = (uint16_t)x;
    coord[npad + k] = (uint16_t)y;
    coord[2 * npad + k] = (uint16_t)z;
}

/* Pull table from the flag: see k_build_nbr for the rule.  s = x - e_j
 * pushes into x if fluid; x bounces if t = x + e_j is solid; when both
 * write, the later in node order wins, i.e. the push iff s's cell index is
 * larger (lexicographic numbering is monotone in the cell index) - or always
 * when s lies in another rank slab and remote_wins is set. */
__global__ void k_nbr_from_flag(const uint32_t *lexbits, const uint32_t *obits,
                                const uint32_t *ooffs, Grid g, int slab,
                                int remote_wins, int halfway, int n, long long npad,
                                uint32_t word_base, uint32_t rest_word,
                                const uint16_t *coord, uint32_t *nbr)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int x = coord[k], y = coord[npad + k], z = coord[2 * npad + k];
    const size_t cx = ((size_t)z * g.ny + y) * g.nx + x;
#pragma unroll
    for (int j = 1; j < Q; j++) {
        int sx = x - ex(j), sy = y - ey(j), sz = z - ez(j);
        int tx = x + ex(j), ty = y + ey(j), tz = z + ez(j);
        sx = sx < 0 ? sx + g.nx : (sx >= g.nx ? sx - g.nx : sx);
        sy = sy < 0 ? sy + g.ny : (sy >= g.ny ? sy - g.ny : sy);
        sz = sz < 0 ? sz + g.nz : (sz >= g.nz ? sz - g.nz : sz);
        tx = tx < 0 ? tx + g.nx : (tx >= g.nx ? tx - g.nx : tx);
        ty = ty < 0 ? ty + g.ny : (ty >= g.ny ? ty - g.ny : ty);
        tz = tz < 0 ? tz + g.nz : (tz >= g.nz ? tz - g.nz : tz);
        const size_t cs = ((size_t)sz * g.ny + sy) * g.nx + sx;
        const size_t ct = ((size_t)tz * g.ny + ty) * g.nx + tx;
        const bool push = bit_at(lexbits, cs);
        const bool bounce = !bit_at(lexbits, ct);
        const bool remote = remote_wins && (sz / slab != z / slab);
        uint32_t word;
        if (halfway)
            word = push ? word_base + rank_in(obits, ooffs, device_key(g, sx, sy, sz))
                        : bounce_word(j, (long long)word_base + k, npad);
        else if (push && (!bounce || remote || cs > cx))
            word = word_base + rank_in(obits, ooffs, device_key(g, sx, sy, sz));
        else if (bounce)
            word = bounce_word(j, (long long)word_base + k, npad);
        else
            word = rest_word;
        nbr[(long long)(j - 1) * npad + k] = word;
    }
}

/* --------------------------------------------------------- sphere pack */

/* Same inside test as plb_sphere_pack (plb_host.c), with round-to-nearest
 * intrinsics so no FMA contraction changes a bit. */
__device__ __forceinline__ double min_image_d(double a, double c, int n)
{
    const double d = fabs(__dsub_rn(a, c));
    const double w = __dsub_rn((double)n, d);
    return d <= w ? d : w;
}

struct Sphere {
    double cx, cy, cz, r;
};

/* one block per sphere: every cell of its bounding box that lies inside
 * takes the sphere's index if it is the first to cover it */
__global__ void k_cover(const Sphere *sp, int base, int count, int nx, int ny,
                        int nz, uint32_t *first)
{
    const int k = blockIdx.x;
    if (k >= count) return;
    const Sphere s = sp[k];
    const double r2 = __dmul_rn(s.r, s.r);
    int x0 = (int)floor(s.cx - s.r) - 1, x1 = (int)ceil(s.cx + s.r) + 1;
    int y0 = (int)floor(s.cy - s.r) - 1, y1 = (int)ceil(s.cy + s.r) + 1;
    int z0 = (int)floor(s.cz - s.r) - 1, z1 = (int)ceil(s.cz + s.r) + 1;
    if (x1 - x0 + 1 > nx) x1 = x0 + nx - 1;
    if (y1 - y0 + 1 > ny) y1 = y0 + ny - 1;
    if (z1 - z0 + 1 > nz) z1 = z0 + nz - 1;
    const int wx = x1 - x0 + 1, wy = y1 - y0 + 1, wz = z1 - z0 + 1;
    const long long vol = (long long)wx * wy * wz;
    const uint32_t idx = (uint32_t)(base + k);
    for (long long t = threadIdx.x; t < vol; t += blockDim.x) {
        const int X = x0 + (int)(t % wx);
        const int Y = y0 + (int)((t / wx) % wy);
        const int Z = z0 + (int)(t / ((long long)wx * wy));
        const int x = ((X % nx) + nx) % nx;
        const int y = ((Y % ny) + ny) % ny;
        const int z = ((Z % nz) + nz) % nz;
        const double dx = min_image_d((double)x, s.cx, nx);
        const double dy = min_image_d((double)y, s.cy, ny);
        const double dz = min_image_d((double)z, s.cz, nz);
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                    __dmul_rn(dz, dz));
        if (d2 <= r2) atomicMin(first + ((size_t)z * ny + y) * nx + x, idx);
    }
}

/* hist[f - lo] += 1 for every cell first covered by sphere f in [lo, hi) */
__global__ void k_first_hist(const uint32_t *first, size_t cells, uint32_t lo,
                             uint32_t hi, unsigned long long *hist)
{
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    const uint32_t f = first[c];
    if (f >= lo && f < hi) atomicAdd(hist + (f - lo), 1ull);
}

__global__ void k_popc_words(const uint32_t *bits, uint32_t *cnt, size_t m)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) cnt[k] = __popc(bits[k]);
}

__global__ void k_flag_from_first(const uint32_t *first, size_t cells,
                                  uint32_t nsph, uint8_t *flag)
{
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    flag[c] = first[c] < nsph ? 0 : 1;
}

}  // namespace plb

using namespace plb;

/* ------------------------------------------------------ host interfaces */

namespace plb {

static unsigned gsz(size_t n, int b) { return (unsigned)((n + b - 1) / b); }

static int ceil_log2i(int v)
{
    int b = 0;
    while ((1LL << b) < v) b++;
    return b;
}

/* splitmix64 (Steele, Lea & Flood 2014), the same stream as plb_host.c */
static uint64_t sm64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static double u01(uint64_t *s) { return (double)(sm64(s) >> 11) * 0x1.0p-53; }

#define CKG(call)                                                             \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) {                                              \
            fprintf(stderr, "porelb_gpu: %s failed: %s\n", #call,             \
                    cudaGetErrorString(e_));                                  \
            rc = e_ == cudaErrorMemoryAllocation ? PLB_ERR_NOMEM : PLB_ERR_CUDA; \
            goto done;                                                        \
        }                                                                     \
    } while (0)

int sphere_pack_device(uint64_t seed, int nx, int ny, int nz, double rmin,
                       double rmax, double porosity, uint8_t *dflag,
                       int *num_spheres, double *porosity_out, cudaStream_t st)
{
    const size_t cells = (size_t)nx * ny * nz;
    const double total = (double)cells;
    int rc = PLB_OK;
    uint32_t *first = nullptr;
    Sphere *dsp = nullptr;
    unsigned long long *hist = nullptr;
    Sphere *hsp = nullptr;
    unsigned long long *hh = nullptr;
    uint64_t state = seed;
    long long made = 0, ns = -1;
    long long fluid = (long long)cells;
    /* expected sphere count for the target porosity, from the mean volume */
    const double rm = 0.5 * (rmin + rmax);
    const double v = 4.18879020478639 * rm * rm * rm;
    long long chunk = (long long)(-log(porosity > 1e-6 ? porosity : 1e-6) * total / v * 1.3) + 64;
    if (chunk > 4000000) chunk = 4000000;
    CKG(plb_cuda_malloc(&first, cells * 4));
    CKG(cudaMemsetAsync(first, 0xff, cells * 4, st));
    CKG(plb_cuda_malloc(&dsp, sizeof(Sphere) * (size_t)chunk));
    CKG(plb_cuda_malloc(&hist, sizeof(unsigned long long) * (size_t)chunk));
    hsp = (Sphere *)malloc(sizeof(Sphere) * (size_t)chunk);
    hh = (unsigned long long *)malloc(sizeof(unsigned long long) * (size_t)chunk);
    if (!hsp || !hh) { rc = PLB_ERR_NOMEM; goto done; }
    if (!((double)fluid / total > porosity)) ns = 0;
    while (ns < 0) {
        if (made > 100000000LL) { rc = PLB_ERR_ARG; goto done; }
        for (long long k = 0; k < chunk; k++) {
            hsp[k].cx = u01(&state) * nx;
            hsp[k].cy = u01(&state) * ny;
            hsp[k].cz = u01(&state) * nz;
            hsp[k].r = rmin + (rmax - rmin) * u01(&state);
        }
        CKG(cudaMemcpyAsync(dsp, hsp, sizeof(Sphere) * (size_t)chunk, cudaMemcpyHostToDevice, st));
        k_cover<<<(unsigned)chunk, 256, 0, st>>>(dsp, (int)made, (int)chunk, nx, ny, nz, first);
        CKG(cudaGetLastError());
        /* cells first covered by each sphere of this chunk */
        CKG(cudaMemsetAsync(hist, 0, sizeof(unsigned long long) * (size_t)chunk, st));
        k_first_hist<<<gsz(cells, 256), 256, 0, st>>>(first, cells, (uint32_t)made,
                                                     (uint32_t)(made + chunk), hist);
        CKG(cudaGetLastError());
        CKG(cudaMemcpyAsync(hh, hist, sizeof(unsigned long long) * (size_t)chunk, cudaMemcpyDeviceToHost, st));
        CKG(cudaStreamSynchronize(st));
        for (long long k = 0; k < chunk && ns < 0; k++) {
            fluid -= (long long)hh[k];
            if (!((double)fluid / total > porosity)) ns = made + k + 1;
        }
        made += chunk;
        if (ns < 0 && made + chunk > 0x7fffffffLL) { rc = PLB_ERR_ARG; goto done; }
    }
    k_flag_from_first<<<gsz(cells, 256), 256, 0, st>>>(first, cells, (uint32_t)ns, dflag);
    CKG(cudaGetLastError());
    CKG(cudaStreamSynchronize(st));
    if (num_spheres) *num_spheres = (int)ns;
    if (porosity_out) *porosity_out = (double)fluid / total;
done:
    cudaStreamSynchronize(st);
    cudaFree(first);
    cudaFree(dsp);
    cudaFree(hist);
    free(hsp);
    free(hh);
    return rc;
}

/* Lexicographic ranks of the fluid cells of a device flag grid.
 * lexbits/lexoffs: (cells+31)/32 words each.  *n receives the fluid count,
 * slab_start[num_p] the first node of every z slab. */
int flag_rank(const uint8_t *dflag, int nx, int ny, int nz, int num_p,
              uint32_t *lexbits, uint32_t *lexoffs, int *n, int *slab_start,
              cudaStream_t st)
{
    const size_t cells = (size_t)nx * ny * nz;
    const size_t words = (cells + 31) / 32;
    int rc = PLB_OK;
    unsigned *bad = nullptr;
    uint32_t *cnt = nullptr;
    unsigned hbad = 0;
    CKG(plb_cuda_malloc(&bad, 4));
    CKG(plb_cuda_malloc(&cnt, words * 4));
    CKG(cudaMemsetAsync(bad, 0, 4, st));
    k_flag_bits<<<gsz(words, 256), 256, 0, st>>>(dflag, cells, lexbits, cnt, words, bad);
    CKG(cudaGetLastError());
    rc = scan_words(cnt, lexoffs, words, st);
    if (rc != PLB_OK) goto done;
    {
        uint32_t last_off = 0, last_cnt = 0;
        CKG(cudaMemcpyAsync(&last_off, lexoffs + words - 1, 4, cudaMemcpyDeviceToHost, st));
        CKG(cudaMemcpyAsync(&last_cnt, cnt + words - 1, 4, cudaMemcpyDeviceToHost, st));
        CKG(cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, st));
        CKG(cudaStreamSynchronize(st));
        if (hbad) { rc = PLB_ERR_ARG; goto done; }
        const long long total = (long long)last_off + last_cnt;
        if (total >= kMaxNodes) { rc = PLB_ERR_ARG; goto done; }
        *n = (int)total;
        /* slab starts: rank of the first cell of each slab (cell index is a
         * multiple of 32 only when the plane is; count the remainder) */
        const int slab = nz / num_p;
        for (int p = 0; p < num_p; p++) {
            const size_t c = (size_t)p * slab * nx * ny;
            if (c >= cells) { slab_start[p] = *n; continue; }
            uint32_t off = 0, word = 0;
            CKG(cudaMemcpyAsync(&off, lexoffs + c / 32, 4, cudaMemcpyDeviceToHost, st));
            CKG(cudaMemcpyAsync(&word, lexbits + c / 32, 4, cudaMemcpyDeviceToHost, st));
            CKG(cudaStreamSynchronize(st));
            slab_start[p] = (int)(off + __builtin_popcount(word & ((1u << (c & 31)) - 1u)));
        }
    }
done:
    cudaStreamSynchronize(st);
    cudaFree(bad);
    cudaFree(cnt);
    return rc;
}

/* Morton (or reference) order, permutation, coordinates and pull table of
 * the fluid cells of a device flag grid, ranked by flag_rank. */
int flag_tables(const uint8_t *dflag, int nx, int ny, int nz, int num_p,
                int ordering, int remote_wins, int halfway, const uint32_t *lexbits,
                const uint32_t *lexoffs, int n, long long npad, int *perm,
                uint16_t *coord, uint32_t *nbr, uint32_t word_base,
                uint32_t rest_word, cudaStream_t st)
{
    (void)dflag;
    const size_t cells = (size_t)nx * ny * nz;
    Grid g{nx, ny, nz, ceil_log2i(nx), ceil_log2i(ny), ceil_log2i(nz),
           ordering == PLB_ORDER_MORTON};
    const int bits = g.morton ? g.bx + g.by + g.bz : 0;
    if (bits > 40) return PLB_ERR_ARG;
    const size_t space = g.morton ? ((size_t)1 << bits) : cells;
    const size_t owords = (space + 31) / 32;
    int rc = PLB_OK;
    uint32_t *obits = nullptr, *ooffs = nullptr, *ocnt = nullptr;
    if (n == 0) return PLB_OK;
    CKG(plb_cuda_malloc(&obits, owords * 4));
    CKG(plb_cuda_malloc(&ooffs, owords * 4));
    CKG(plb_cuda_malloc(&ocnt, owords * 4));
    CKG(cudaMemsetAsync(obits, 0, owords * 4, st));
    k_mark_order<<<gsz(cells, 256), 256, 0, st>>>(lexbits, g, cells, obits);
    CKG(cudaGetLastError());
    k_popc_words<<<gsz(owords, 256), 256, 0, st>>>(obits, ocnt, owords);
    CKG(cudaGetLastError());
    rc = scan_words(ocnt, ooffs, owords, st);
    if (rc != PLB_OK) goto done;
    k_assign_from_flag<<<gsz(cells, 256), 256, 0, st>>>(lexbits, lexoffs, obits, ooffs, g,
                                                       cells, n, npad, perm, coord);
    CKG(cudaGetLastError());
    k_nbr_from_flag<<<gsz((size_t)n, 128), 128, 0, st>>>(lexbits, obits, ooffs, g, nz / num_p,
                                                        remote_wins, halfway, n, npad,
                                                        word_base, rest_word, coord, nbr);
    CKG(cudaGetLastError());
    CKG(cudaStreamSynchronize(st));
done:
    cudaStreamSynchronize(st);
    cudaFree(obits);
    cudaFree(ooffs);
    cudaFree(ocnt);
    return rc;
}

}  // namespace plb
