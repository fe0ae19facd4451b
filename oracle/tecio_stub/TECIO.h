/*
 * TECIO.h - no-op stand-in for the Tecplot I/O library, used only to compile
 * the reference's postprocess.c slice modes into the test oracle.  The
 * Tecplot (A) mode is not exercised.  TEST INFRASTRUCTURE ONLY.
 */
#ifndef ORACLE_TECIO_STUB_H_
#define ORACLE_TECIO_STUB_H_
typedef int INTEGER4;
static INTEGER4 TECINI112() { return 0; }
static INTEGER4 TECZNE112() { return 0; }
static INTEGER4 TECDAT112() { return 0; }
static INTEGER4 TECEND112() { return 0; }
#endif
