/*
 * plb_host.c - host-side parts of the C ABI: the node-table builder that
 * replaces porelb's preprocess (build_V / save_V), the V.bin reader of
 * alloc_memory, the check_V bounds test and the sphere-pack geometry source.
 *
 * Built with -ffp-contract=off: the sphere test must give the same answer
 * here and in the device generator.
 */
#include "porelb_gpu.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* D3Q19 velocities in the reference order (porelb.h:10-34). */
static const int kE[PLB_Q][3] = {
    {0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
    {0, 0, 1},  {0, 0, -1},  {0, 1, 1},  {0, -1, -1}, {0, -1, 1},
    {0, 1, -1}, {-1, 0, -1}, {1, 0, 1},  {-1, 0, 1}, {1, 0, -1},
    {-1, 1, 0}, {1, -1, 0},  {-1, -1, 0}, {1, 1, 0}};

void plb_default_params(plb_params *p)
{
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->tau = 0.8;       /* porelb.c:87 */
    p->force_x = 1e-3;  /* porelb.c:91 */
    p->precision = PLB_FP64_EXACT;
    p->ordering = PLB_ORDER_AUTO;
    p->halo = PLB_HALO_AUTO;
    p->block_size = 0;
    p->device = 0;
    p->boundary = PLB_BOUNDARY_REFERENCE;
}

const char *plb_status_string(int s)
{
    switch (s) {
    case PLB_OK: return "ok";
    case PLB_ERR_ARG: return "invalid argument";
    case PLB_ERR_IO: return "file i/o error";
    case PLB_ERR_TABLE: return "node table fails the bounds check";
    case PLB_ERR_CUDA: return "CUDA error or no CUDA device";
    case PLB_ERR_NOMEM: return "out of memory";
    case PLB_ERR_DENSITY: return "density guard tripped (rho > 1.2 or rho < 0.5)";
    case PLB_ERR_NUMP: return "num_p inconsistent with the node table";
    case PLB_ERR_STATE: return "call out of order";
    default: return "unknown status";
    }
}

/* ------------------------------------------------------------ node table */

/* The table follows build_V (preprocess.c:29-164): fluid nodes (flag == 1)
 * numbered in x-fastest lexicographic order, rank = z / (nz/num_p), each
 * record placed at v_sub_start[rank] + its position within the rank.
 * Neighbour slot d describes (x,y,z)+e[d+1] with periodic wrap.  A zero flag
 * gives SOLID; the record is a running temporary in the reference, so a SOLID
 * slot keeps the id/pid written at that slot for the last node whose
 * neighbour there was not solid (zero before any such node).  Any nonzero
 * flag gives FLUID/EXTERN with that cell's fluid number, which is 0 for
 * flag values other than 1 (the reference's calloc'd map). */
int plb_build_table(const uint8_t *flag, int nx, int ny, int nz, int num_p,
                    plb_node_info *out, int *num_node, int *v_sub_start)
{
    if (!flag || !num_node || nx <= 0 || ny <= 0 || nz <= 0 || num_p <= 0 ||
        num_p > nz || nz % num_p != 0 || nx > 65536 || ny > 65536 ||
        nz > 65536 || num_p > 65535)
        return PLB_ERR_ARG;
    const size_t plane = (size_t)nx * ny;
    const size_t cells = plane * (size_t)nz;
    const int slab = nz / num_p;

    /* Per-slab fluid counts; fluid numbering is slab-major anyway because a
     * slab is a contiguous range of z planes. */
    long long *slab_count = (long long *)calloc((size_t)num_p, sizeof(long long));
    if (!slab_count) return PLB_ERR_NOMEM;
    long long total = 0;
    for (int z = 0; z < nz; z++) {
        const uint8_t *row = flag + (size_t)z * plane;
        long long c = 0;
        for (size_t k = 0; k < plane; k++) c += (row[k] == 1);
        slab_count[z / slab] += c;
        total += c;
    }
    if (total > 0x7fffffffLL) {
        free(slab_count);
        return PLB_ERR_ARG;
    }
    *num_node = (int)total;
    if (!out) {
        if (v_sub_start) {
            long long s = 0;
            for (int p = 0; p < num_p; p++) {
                v_sub_start[p] = (int)s;
                s += slab_count[p];
            }
        }
        free(slab_count);
        return PLB_OK;
    }

    /* fluid number of every cell (0 for non-fluid cells, as the reference) */
    uint32_t *num = (uint32_t *)malloc(cells * sizeof(uint32_t));
    int *start = (int *)malloc(sizeof(int) * ((size_t)num_p + 1));
    if (!num || !start) {
        free(num); free(start); free(slab_count);
        return PLB_ERR_NOMEM;
    }
    {
        uint32_t n = 0;
        for (size_t k = 0; k < cells; k++) {
            num[k] = (flag[k] == 1) ? n : 0u;
            n += (flag[k] == 1);
        }
    }
    long long s = 0;
    for (int p = 0; p < num_p; p++) {
        start[p] = (int)s;
        s += slab_count[p];
    }
    start[num_p] = (int)s;
    if (v_sub_start) memcpy(v_sub_start, start, sizeof(int) * (size_t)num_p);

    /* Since fluid numbering is lexicographic and slabs are z ranges, the
     * position within the rank is (global number - start[rank]) and the
     * output index equals the global number. */
    plb_node_info cur;
    memset(&cur, 0, sizeof(cur));
    size_t g = 0;
    for (int z = 0; z < nz; z++) {
        const int p = z / slab;
        for (int y = 0; y < ny; y++) {
            for (int x = 0; x < nx; x++) {
                const size_t k = ((size_t)z * ny + y) * nx + x;
                if (flag[k] != 1) continue;
                cur.x = (uint16_t)x;
                cur.y = (uint16_t)y;
                cur.z = (uint16_t)z;
                for (int d = 0; d < PLB_Q - 1; d++) {
                    int xs = x + kE[d + 1][0], ys = y + kE[d + 1][1],
                        zs = z + kE[d + 1][2];
                    xs = xs < 0 ? xs + nx : (xs >= nx ? xs - nx : xs);
                    ys = ys < 0 ? ys + ny : (ys >= ny ? ys - ny : ys);
                    zs = zs < 0 ? zs + nz : (zs >= nz ? zs - nz : zs);
                    const size_t kn = ((size_t)zs * ny + ys) * nx + xs;
                    plb_neighbor_info *nb = &cur.nb_info[d];
                    if (flag[kn] == 0) {
                        nb->node_type = PLB_TYPE_SOLID;
                        continue;
                    }
                    const uint32_t gn = num[kn];
                    /* rank of the neighbour's fluid number */
                    int pn = zs / slab;
                    if (flag[kn] != 1) {
                        /* the reference looks up fluid number 0 */
                        int q = 0;
                        while (q + 1 < num_p && start[q + 1] <= 0) q++;
                        pn = q;
                    }
                    nb->node_pid = (uint16_t)pn;
                    nb->node_id = gn - (uint32_t)start[pn];
                    nb->node_type =
                        (uint8_t)(pn == p ? PLB_TYPE_FLUID : PLB_TYPE_EXTERN);
                }
                out[g++] = cur;
            }
        }
    }
    free(num);
    free(start);
    free(slab_count);
    return PLB_OK;
}

int plb_check_table(const plb_node_info *V, int num_node, int nx, int ny,
                    int nz, int num_p, const int *v_sub_start)
{
    if (!V && num_node > 0) return PLB_ERR_ARG;
    if (num_node < 0 || num_p <= 0 || !v_sub_start) return PLB_ERR_ARG;
    for (int p = 0; p < num_p; p++) {
        int lo = v_sub_start[p];
        int hi = (p + 1 < num_p) ? v_sub_start[p + 1] : num_node;
        if (lo < 0 || hi < lo || hi > num_node) return PLB_ERR_NUMP;
    }
    if (v_sub_start[0] != 0) return PLB_ERR_NUMP;
    int p = 0;
    for (int i = 0; i < num_node; i++) {
        while (p + 1 < num_p && i >= v_sub_start[p + 1]) p++;
        const plb_node_info *r = &V[i];
        if (r->x >= nx || r->y >= ny || r->z >= nz) return PLB_ERR_TABLE;
        for (int d = 0; d < PLB_Q - 1; d++) {
            const plb_neighbor_info *nb = &r->nb_info[d];
            if (nb->node_type == PLB_TYPE_SOLID) continue;
            if (nb->node_type > PLB_TYPE_EXTERN) return PLB_ERR_TABLE;
            int q = nb->node_type == PLB_TYPE_FLUID ? p : nb->node_pid;
            if (nb->node_type == PLB_TYPE_EXTERN && (q >= num_p || q == p))
                return PLB_ERR_TABLE;
            if (nb->node_type == PLB_TYPE_FLUID && nb->node_pid != p)
                return PLB_ERR_TABLE;
            int hi = (q + 1 < num_p) ? v_sub_start[q + 1] : num_node;
            if ((long long)v_sub_start[q] + nb->node_id >= hi)
                return PLB_ERR_TABLE;
        }
    }
    return PLB_OK;
}

/* ------------------------------------------------------------------ V.bin */

int plb_write_vbin(const char *path, const plb_node_info *V, int num_node,
                   int num_p, int nx, int ny, int nz, const int *v_sub_start)
{
    if (!path || num_node < 0 || num_p <= 0 || !v_sub_start ||
        (num_node > 0 && !V))
        return PLB_ERR_ARG;
    FILE *fp = fopen(path, "wb");
    if (!fp) return PLB_ERR_IO;
    int32_t hdr[5] = {num_node, num_p, nx, ny, nz};
    int ok = fwrite(hdr, sizeof(int32_t), 5, fp) == 5 &&
             fwrite(v_sub_start, sizeof(int32_t), (size_t)num_p, fp) ==
                 (size_t)num_p &&
             fwrite(V, sizeof(plb_node_info), (size_t)num_node, fp) ==
                 (size_t)num_node;
    if (fclose(fp) != 0) ok = 0;
    return ok ? PLB_OK : PLB_ERR_IO;
}

int plb_read_vbin_header(const char *path, int *num_node, int *num_p, int *nx,
                         int *ny, int *nz)
{
    if (!path) return PLB_ERR_ARG;
    FILE *fp = fopen(path, "rb");
    if (!fp) return PLB_ERR_IO;
    int32_t hdr[5];
    size_t got = fread(hdr, sizeof(int32_t), 5, fp);
    fclose(fp);
    if (got != 5) return PLB_ERR_IO;
    if (hdr[0] < 0 || hdr[1] <= 0 || hdr[2] <= 0 || hdr[3] <= 0 || hdr[4] <= 0)
        return PLB_ERR_IO;
    if (num_node) *num_node = hdr[0];
    if (num_p) *num_p = hdr[1];
    if (nx) *nx = hdr[2];
    if (ny) *ny = hdr[3];
    if (nz) *nz = hdr[4];
    return PLB_OK;
}

int plb_read_vbin(const char *path, plb_node_info *V, int *v_sub_start)
{
    if (!path || !v_sub_start) return PLB_ERR_ARG;
    FILE *fp = fopen(path, "rb");
    if (!fp) return PLB_ERR_IO;
    int32_t hdr[5];
    int st = PLB_OK;
    if (fread(hdr, sizeof(int32_t), 5, fp) != 5 || hdr[0] < 0 || hdr[1] <= 0) {
        st = PLB_ERR_IO;
    } else if (fread(v_sub_start, sizeof(int32_t), (size_t)hdr[1], fp) !=
               (size_t)hdr[1]) {
        st = PLB_ERR_IO;
    } else if (hdr[0] > 0 &&
               (!V || fread(V, sizeof(plb_node_info), (size_t)hdr[0], fp) !=
                          (size_t)hdr[0])) {
        st = V ? PLB_ERR_IO : PLB_ERR_ARG;
    }
    fclose(fp);
    return st;
}

/* ------------------------------------------------------------ sphere pack */

static uint64_t splitmix64_next(uint64_t *state)
{
    /* splitmix64 (Steele, Lea & Flood, OOPSLA 2014) */
    uint64_t z = (*state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double uniform01(uint64_t *state)
{
    return (double)(splitmix64_next(state) >> 11) * 0x1.0p-53;
}

/* periodic minimum-image distance along one axis */
static double min_image(double a, double c, int n)
{
    double d = fabs(a - c);
    double w = (double)n - d;
    return d <= w ? d : w;
}

int plb_sphere_pack(uint64_t seed, int nx, int ny, int nz, double rmin,
                    double rmax, double porosity, uint8_t *flag,
                    int *num_spheres, double *porosity_out)
{
    if (!flag || nx <= 0 || ny <= 0 || nz <= 0 || !(rmin > 0.0) ||
        rmax < rmin || !(porosity >= 0.0) || !(porosity <= 1.0))
        return PLB_ERR_ARG;
    const size_t cells = (size_t)nx * ny * nz;
    memset(flag, 1, cells);
    size_t fluid = cells;
    uint64_t st = seed;
    int ns = 0;
    const double total = (double)cells;
    /* a sphere can never be required beyond this many draws */
    const long max_spheres = 100000000L;
    while ((double)fluid / total > porosity && ns < max_spheres) {
        const double cx = uniform01(&st) * nx;
        const double cy = uniform01(&st) * ny;
        const double cz = uniform01(&st) * nz;
        const double r = rmin + (rmax - rmin) * uniform01(&st);
        const double r2 = r * r;
        ns++;
        const int x0 = (int)floor(cx - r), x1 = (int)ceil(cx + r);
        const int y0 = (int)floor(cy - r), y1 = (int)ceil(cy + r);
        const int z0 = (int)floor(cz - r), z1 = (int)ceil(cz + r);
        const int xe = (x1 - x0 + 1 > nx) ? x0 + nx - 1 : x1;
        const int ye = (y1 - y0 + 1 > ny) ? y0 + ny - 1 : y1;
        const int ze = (z1 - z0 + 1 > nz) ? z0 + nz - 1 : z1;
        for (int Z = z0; Z <= ze; Z++) {
            const int z = ((Z % nz) + nz) % nz;
            const double dz = min_image((double)z, cz, nz);
            for (int Y = y0; Y <= ye; Y++) {
                const int y = ((Y % ny) + ny) % ny;
                const double dy = min_image((double)y, cy, ny);
                uint8_t *row = flag + ((size_t)z * ny + y) * nx;
                for (int X = x0; X <= xe; X++) {
                    const int x = ((X % nx) + nx) % nx;
                    const double dx = min_image((double)x, cx, nx);
                    const double d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 <= r2 && row[x]) {
                        row[x] = 0;
                        fluid--;
                    }
                }
            }
        }
    }
    if (num_spheres) *num_spheres = ns;
    if (porosity_out) *porosity_out = (double)fluid / total;
    return PLB_OK;
}

/* FP64 constants of the collision, in the reference's operation order; this
 * file is compiled without FMA contraction so they are the reference's bits
 * on every host architecture. */
void plb_host_constants(double tau, double force, double *omega, double *om1,
                        double *k3, double *half_force, double *nu)
{
    const double w = 1.0 / tau;        /* porelb.c:88 */
    *omega = w;
    *om1 = 1.0 - w;                    /* (1.0-omega), porelb.c:361 */
    *k3 = (1.0 - 0.5 * w) * 3.0;       /* (1.0-0.5*omega)*3.0, porelb.c:362 */
    *half_force = 0.5 * force;         /* porelb.c:348 */
    if (nu) *nu = 1.0 / 3.0 * (tau - 0.5); /* porelb.c:89 */
}
