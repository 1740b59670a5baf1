/*
 * Minimal stand-in for the configured ATLAS header set, written for the
 * oracle's reference build (oracle/ref_build.sh).  It supplies only what the
 * extracted LU-path routines need: type selection (-DDREAL / -DSREAL), the
 * name-joining macro and a few arithmetic helpers.  TEST INFRASTRUCTURE ONLY.
 */
#ifndef REFSHIM_MISC_H
#define REFSHIM_MISC_H
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <float.h>
#include "atlas_enum.h"
#include "refshim_cblas.h"

#define my_join(a_, b_) a_ ## b_
#define my_str(x_) #x_
#define Mstr(x_) my_str(x_)
#define Mjoin(a_, b_) my_join(a_, b_)
#define Mmin(x_, y_) (((x_) < (y_)) ? (x_) : (y_))
#define Mmax(x_, y_) (((x_) > (y_)) ? (x_) : (y_))
#define Mabs(x_) (((x_) >= 0) ? (x_) : -(x_))
#define ATL_INT int
#define ATL_CINT const int
#define ATL_CSZT const size_t
/* cache-line alignment used by the test library's cache flush */
#define ATL_Cachelen 64
#define ATL_AlignPtr(vp_) ((void *)(ATL_Cachelen + ((((size_t)(vp_)) / ATL_Cachelen) * ATL_Cachelen)))
#define ATL_assert(x_) do { if (!(x_)) { fprintf(stderr, "assert %s\n", #x_); abort(); } } while (0)

#if defined(DREAL)
   #define TREAL
   #define TYPE double
   #define PRE d
   #define ATLAS_PRE d
   #define PATL ATL_d
   #define PATLU ATL_d
   #define ATL_MulBySize(x_) ((x_) << 3)
   #define ATL_DivBySize(x_) ((x_) >> 3)
#elif defined(SREAL)
   #define TREAL
   #define TYPE float
   #define PRE s
   #define ATLAS_PRE s
   #define PATL ATL_s
   #define PATLU ATL_s
   #define ATL_MulBySize(x_) ((x_) << 2)
   #define ATL_DivBySize(x_) ((x_) >> 2)
#else
   #error "define DREAL or SREAL"
#endif
#define SHIFT
/* the serial build's thread multiplier of the cache size (none) */
#define ATL_PTCACHEMUL
#define SCALAR TYPE
#define ATL_rzero ((TYPE)0)
#define ATL_rone ((TYPE)1)
#define ATL_rnone ((TYPE)-1)
#endif
