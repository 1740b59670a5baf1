/* Precision-generic cblas names used by the extracted tester programs, bound
 * to the typed cblas entry points of the library under test (the GPU
 * library), as the reference's testers bind them to the ATLAS build they
 * check.  TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_CBLASTYPEALIAS_H
#define REFSHIM_CBLASTYPEALIAS_H
#include "atlas_misc.h"
#if defined(DREAL)
   #define cblas_trmm cblas_dtrmm
#else
   #define cblas_trmm cblas_strmm
#endif
#endif
