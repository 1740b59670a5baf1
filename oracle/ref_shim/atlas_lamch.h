/* Safe minimum of the working precision (the reference's installer writes the
 * LAPACK dlamch('S') value; for IEEE binary64/binary32 it is DBL_MIN/FLT_MIN).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_LAMCH_H
#define REFSHIM_LAMCH_H
#include <float.h>
#ifdef DREAL
   #define ATL_laSAFMIN DBL_MIN
#else
   #define ATL_laSAFMIN FLT_MIN
#endif
#endif
