/*
 * postprocess_main.c - drop-in replacement of the reference postprocess
 * executable (postprocess.c:87-319):
 *
 *   postprocess.x X|Y|Z n time_list...   ASCII slice files Slice_X_%07d.dat ...
 *   postprocess.x R time_list...         full grid, raw binary full_%07d.raw
 *   postprocess.x A time_list...         Tecplot binary (TECIO) - not
 *                                        available in this build
 *
 * Reads V.bin, flag.bin and every rank's part_%03d_%07d.bin from the working
 * directory and scatters rho, ux, uy, uz onto the nx*ny*nz grid through the
 * node coordinates (postprocess.c:175-214); solid cells stay 0.  The slice
 * files keep the reference's header lines and column formats
 * (postprocess.c:19-85), including its zone sizes and titles.  The last
 * column is the cell flag printed as a double (the reference passes an int
 * to a %e conversion there, which prints an undefined value).
 * R writes int32 nx, ny, nz then rho, ux, uy, uz as nx*ny*nz doubles each.
 *
 * The reference's slice writers loop over the whole time list each time a
 * time's data is loaded (postprocess.c:23-39 inside the loop of :175-306),
 * so every slice file it leaves holds the LAST time's data.  By default each
 * file here holds its own time; with PLB_SLICE_COMPAT=1 in the environment
 * the reference's behaviour is reproduced.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "porelb_gpu.h"

static void usage(void)
{
    printf("Usage: ./postprocess.x  [A|R|X|Y|Z] [n] time_list\n");
    printf("Output 3D full data     : ./postprocess.x R time_list\n");
    printf("Output slice at  X = 20 : ./postprocess.x X 20  time_list\n");
}

static int write_slice(char mode, int n, int tag, int nx, int ny, int nz,
                       const double *rho, const double *u, const double *v,
                       const double *w, const unsigned char *flag)
{
    char name[64];
    snprintf(name, sizeof(name), "Slice_%c_%07d.dat", mode, tag);
    FILE *fp = fopen(name, "w");
    if (!fp) return -1;
    const long plane = (long)nx * ny;
    if (mode == 'X') {
        fprintf(fp, "TITLE = \" X slice at %04d\"\n", n);
        fprintf(fp, "Variables = \"X\", \"Y\", \"Rho\", \"Ux\", \"Uy\", \"Uz\", \"flag\"\n");
        fprintf(fp, "ZONE I = %4d, J = %4d, F=POINT\n", ny, nz);
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++) {
                const long loc = k * plane + (long)j * nx + n;
                fprintf(fp, "%f %f % 21.14e  % 21.14E  % 21.14E  % 21.14E  % 8.1e\n",
                        (double)k, (double)j, rho[loc], u[loc], v[loc], w[loc],
                        (double)flag[loc]);
            }
    } else if (mode == 'Y') {
        fprintf(fp, "TITLE = \" Y slice at %04d\"\n", n);
        fprintf(fp, "Variables = \"X\", \"Y\", \"Rho\", \"Ux\", \"Uy\", \"Uz\", \"flag\"\n");
        fprintf(fp, "ZONE I = %4d, J = %4d, F=POINT\n", nz, nx);
        for (int k = 0; k < nz; k++)
            for (int i = 0; i < nx; i++) {
                const long loc = k * plane + (long)n * nx + i;
                fprintf(fp, "%f %f % 21.14e  % 21.14E  % 21.14E  % 21.14E  % 8.1e\n",
                        (double)k, (double)i, rho[loc], u[loc], v[loc], w[loc],
                        (double)flag[loc]);
            }
    } else {
        /* the reference titles the Z slice "Y slice" (postprocess.c:73) */
        fprintf(fp, "TITLE = \" Y slice at %04d\"\n", n);
        fprintf(fp, "Variables = \"X\", \"Y\", \"Rho\", \"Ux\", \"Uy\", \"Uz\", \"flag\"\n");
        fprintf(fp, "ZONE I = %4d, J = %4d, F=POINT\n", nz, nx);
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const long loc = (long)n * plane + (long)j * nx + i;
                fprintf(fp, "%f %f % 21.14e  % 21.14E  % 21.14E  % 21.14E  % 8.1e\n",
                        (double)j, (double)i, rho[loc], u[loc], v[loc], w[loc],
                        (double)flag[loc]);
            }
    }
    return fclose(fp) == 0 ? 0 : -1;
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        usage();
        return -2;
    }
    const char mode = argv[1][0];
    if (strlen(argv[1]) != 1 || !strchr("ARXYZ", mode)) {
        fprintf(stderr, "Not implemented yet!\n");
        return -3;
    }
    if (mode == 'A') {
        fprintf(stderr, "Tecplot binary output needs the TECIO library, which "
                        "this build does not have; use R (raw) or X/Y/Z.\n");
        return -3;
    }
    const int first = (mode == 'R') ? 2 : 3;
    if (argc < first) {
        usage();
        return -2;
    }
    const int n_slice = (mode == 'R') ? 0 : atoi(argv[2]);
    const char *cenv = getenv("PLB_SLICE_COMPAT");
    const int compat = cenv && cenv[0] == '1';
    const int nt = argc - first;
    printf("Total %d time seriese data\n", nt);

    int num_f, num_p, nx, ny, nz;
    if (plb_read_vbin_header("V.bin", &num_f, &num_p, &nx, &ny, &nz) != PLB_OK) {
        fprintf(stderr, "Node map file openning error!\n");
        return -1;
    }
    printf(">>> Total num of fluid  nodes = %d\n", num_f);
    printf(">>> num_p = %d\n", num_p);
    plb_node_info *V = (plb_node_info *)malloc(sizeof(plb_node_info) * (size_t)(num_f ? num_f : 1));
    int *start = (int *)malloc(sizeof(int) * ((size_t)num_p + 1));
    if (!V || !start || plb_read_vbin("V.bin", V, start) != PLB_OK) {
        fprintf(stderr, "Node map file openning error!\n");
        return -1;
    }
    start[num_p] = num_f;
    if ((mode == 'X' && (n_slice < 0 || n_slice >= nx)) ||
        (mode == 'Y' && (n_slice < 0 || n_slice >= ny)) ||
        (mode == 'Z' && (n_slice < 0 || n_slice >= nz))) {
        fprintf(stderr, "slice index out of range\n");
        return -2;
    }
    const size_t cells = (size_t)nx * ny * nz;
    double *rho = (double *)calloc(cells, sizeof(double));
    double *u = (double *)calloc(cells, sizeof(double));
    double *v = (double *)calloc(cells, sizeof(double));
    double *w = (double *)calloc(cells, sizeof(double));
    unsigned char *flag = (unsigned char *)calloc(cells, 1);
    if (!rho || !u || !v || !w || !flag) {
        fprintf(stderr, "Memory allocating failed!\n");
        return -3;
    }
    FILE *ff = fopen("flag.bin", "rb");
    if (!ff) {
        fprintf(stderr, "Flag file openning error!\n");
        return -1;
    }
    if (fread(flag, 1, cells, ff) != cells) {
        fprintf(stderr, "Flag file reading error!\n");
        fclose(ff);
        return -1;
    }
    fclose(ff);

    for (int it = 0; it < nt; it++) {
        const int tag = atoi(argv[first + it]);
        for (int p = 0; p < num_p; p++) {
            char name[64];
            snprintf(name, sizeof(name), "part_%03d_%07d.bin", p, tag);
            FILE *fp = fopen(name, "rb");
            if (!fp) {
                fprintf(stderr, "Part file openning error!\n");
                return -1;
            }
            const int N = start[p + 1] - start[p];
            double *buf = (double *)malloc(sizeof(double) * 4 * (size_t)(N ? N : 1));
            if (!buf || fread(buf, sizeof(double), 4 * (size_t)N, fp) != 4 * (size_t)N) {
                fprintf(stderr, "Part file reading error!\n");
                fclose(fp);
                return -1;
            }
            fclose(fp);
            for (int k = 0; k < N; k++) {
                const plb_node_info *r = &V[start[p] + k];
                const size_t loc = ((size_t)r->z * ny + r->y) * nx + r->x;
                rho[loc] = buf[k];
                u[loc] = buf[N + k];
                v[loc] = buf[2 * (size_t)N + k];
                w[loc] = buf[3 * (size_t)N + k];
            }
            free(buf);
        }
        if (mode == 'R') {
            char name[64];
            snprintf(name, sizeof(name), "full_%07d.raw", tag);
            FILE *fp = fopen(name, "wb");
            if (!fp) return -3;
            int hdr[3] = {nx, ny, nz};
            int ok = fwrite(hdr, sizeof(int), 3, fp) == 3 &&
                     fwrite(rho, sizeof(double), cells, fp) == cells &&
                     fwrite(u, sizeof(double), cells, fp) == cells &&
                     fwrite(v, sizeof(double), cells, fp) == cells &&
                     fwrite(w, sizeof(double), cells, fp) == cells;
            if (fclose(fp) != 0 || !ok) return -3;
        } else if (compat) {
            for (int k = 0; k < nt; k++)
                if (write_slice(mode, n_slice, atoi(argv[first + k]), nx, ny, nz, rho, u, v,
                                w, flag) != 0)
                    return -3;
        } else if (write_slice(mode, n_slice, tag, nx, ny, nz, rho, u, v, w, flag) != 0) {
            return -3;
        }
    }
    free(rho); free(u); free(v); free(w); free(flag);
    free(V); free(start);
    return 0;
}
