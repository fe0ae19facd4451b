/*
 * ref_pre_harness.c - exposes the reference's build_V, compiled from the
 * reference's own preprocess.c (included below from the reference tree), for
 * the test oracle.  TEST INFRASTRUCTURE ONLY; built by oracle/Makefile into
 * oracle/_ref/.
 */
#include <string.h>

#define main preprocess_reference_main
#include "preprocess.c"
#undef main

/* Runs build_V (preprocess.c:29-164) on flag_path and copies the result.
 * out receives num_node NODE_INFO records (may be NULL to query the count);
 * v_sub_start receives num_p ints.  Returns num_node. */
int ref_build_v(const char *flag_path, int nx, int ny, int nz, int num_p,
                void *out, int *v_sub_start)
{
    V_DESC d = build_V((unsigned short)num_p, nx, ny, nz, (char *)flag_path);
    if (out) memcpy(out, d.node_info, sizeof(NODE_INFO) * (size_t)d.num_node);
    if (v_sub_start) memcpy(v_sub_start, d.V_sub_start, sizeof(int) * (size_t)num_p);
    int n = d.num_node;
    free_v_desc(&d);
    return n;
}

/* Runs save_V (preprocess.c:166-193) on a table built by build_V. */
int ref_build_and_save_v(const char *flag_path, int nx, int ny, int nz,
                         int num_p, const char *vbin_path)
{
    V_DESC d = build_V((unsigned short)num_p, nx, ny, nz, (char *)flag_path);
    save_V(&d, (char *)vbin_path);
    int n = d.num_node;
    free_v_desc(&d);
    return n;
}
