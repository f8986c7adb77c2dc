/*
 * ref_prelude.h -- definitions the extracted reference hot path needs (test only).
 *
 * oracle/build_ref.py builds oracle/_ref/ref_hotpath.c from this prelude plus the
 * reference's own force, integrator and sort functions (src/c/nsphere.c, line ranges
 * listed in build_ref.py).  Those functions use a handful of macros and globals that
 * live elsewhere in nsphere.c (which needs GSL and FFTW, absent here); this header
 * supplies them so the unmodified function bodies compile alone:
 *   - the unit macros of nsphere.c:364-373 become run-time values so the harness
 *     can run in G = M = 1 units (VEL_CONV_SQ * G_CONST == the G argument);
 *   - CLEAN_EXIT (nsphere.c:289-298) exits without the snapshot cleanup;
 *   - g_defaultSortAlg (nsphere.c:2495) is settable by the harness.
 */
#ifndef NSG_REF_PRELUDE_H
#define NSG_REF_PRELUDE_H
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static double ref_G_value = 1.0;
static double ref_halo_mass = 1.0;

#define PI 3.14159265358979323846
#define G_CONST ref_G_value
#define HALO_MASS ref_halo_mass
#define VEL_CONV_SQ 1.0
#define sqr(x) ((x) * (x))
#define cube(x) ((x) * (x) * (x))
#define CLEAN_EXIT(code) exit(code)

static const char *g_defaultSortAlg = "quadsort";
#endif
