/*
 * ref_post_harness.c - exposes the reference's postprocess main, compiled
 * from the reference's own postprocess.c (included below from the reference
 * tree) with a no-op TECIO header, for the slice-file parity test.
 * TEST INFRASTRUCTURE ONLY; built by oracle/Makefile into oracle/_ref/.
 */
#include <unistd.h>

#define main postprocess_reference_main
#include "postprocess.c"
#undef main

/* Run the reference postprocess in workdir with argv (argv[0] included). */
int ref_postprocess(const char *workdir, int argc, char **argv)
{
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) return -1;
    if (chdir(workdir) != 0) return -1;
    int rc = postprocess_reference_main(argc, argv);
    if (chdir(cwd) != 0) return -1;
    return rc;
}
