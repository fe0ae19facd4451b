/*
 * preprocess_main.c - drop-in replacement of the reference preprocess
 * executable (preprocess.c:195-204, "preprocess.x np").
 *
 * Reads flag.bin (uint8 [z][y][x], 1 fluid, 0 solid) and writes V.bin.  The
 * reference hard-codes a 400^3 grid and both file names; they are the
 * defaults here:  preprocess.x np [nx ny nz] [flag.bin] [V.bin]
 */
#include <stdio.h>
#include <stdlib.h>

#include "porelb_gpu.h"

int main(int argc, char **argv)
{
    if (argc != 2 && argc != 5 && argc != 6 && argc != 7) {
        fprintf(stderr, "Error, usage: ./preprocess.x np [nx ny nz] [flag.bin] [V.bin]\n");
        return -1;
    }
    int num_p = atoi(argv[1]);
    int nx = 400, ny = 400, nz = 400;
    const char *flag_path = "flag.bin", *vbin = "V.bin";
    if (argc >= 5) {
        nx = atoi(argv[2]);
        ny = atoi(argv[3]);
        nz = atoi(argv[4]);
    }
    if (argc >= 6) flag_path = argv[5];
    if (argc >= 7) vbin = argv[6];
    size_t cells = (size_t)nx * ny * nz;
    unsigned char *flag = (unsigned char *)malloc(cells ? cells : 1);
    if (!flag) {
        fprintf(stderr, "Memory allocating failed!\n");
        return -3;
    }
    FILE *fp = fopen(flag_path, "rb");
    if (!fp) {
        fprintf(stderr, "flag data file opening error!\n");
        return -1;
    }
    if (fread(flag, 1, cells, fp) != cells) {
        fprintf(stderr, "flag data file reading error!\n");
        fclose(fp);
        return -2;
    }
    fclose(fp);
    int n = 0;
    int *vs = (int *)malloc(sizeof(int) * (size_t)(num_p > 0 ? num_p : 1));
    int rc = plb_build_table(flag, nx, ny, nz, num_p, NULL, &n, vs);
    if (rc != PLB_OK) {
        fprintf(stderr, "preprocess: %s\n", plb_status_string(rc));
        return -3;
    }
    printf("num_nodes = %d\n", n);
    plb_node_info *V = (plb_node_info *)malloc(sizeof(plb_node_info) * (size_t)(n ? n : 1));
    if (!V) {
        fprintf(stderr, "Memory allocating failed!\n");
        return -3;
    }
    rc = plb_build_table(flag, nx, ny, nz, num_p, V, &n, vs);
    if (rc == PLB_OK) rc = plb_write_vbin(vbin, V, n, num_p, nx, ny, nz, vs);
    if (rc != PLB_OK) {
        fprintf(stderr, "File writing failed\n");
        return -1;
    }
    printf("V.bin written %ld Bytes\n", (long)n * (long)sizeof(plb_node_info));
    printf("NODE_INFO_size: %ld Bytes\n", (long)sizeof(plb_node_info));
    free(V);
    free(vs);
    free(flag);
    return 0;
}
