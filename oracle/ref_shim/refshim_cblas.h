/* Generic-name BLAS calls of the extracted LU routines, routed to the
 * reference BLAS (ATL_?ref*) by ref_glue.c.  TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_CBLAS_H
#define REFSHIM_CBLAS_H
#include "atlas_enum.h"   /* the reference's cblas enum values */

void refshim_dgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE, int, int, int,
                   double, const double*, int, const double*, int, double, double*, int);
void refshim_sgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE, int, int, int,
                   float, const float*, int, const float*, int, float, float*, int);
void refshim_dtrsm(enum CBLAS_ORDER, enum CBLAS_SIDE, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE,
                   enum CBLAS_DIAG, int, int, double, const double*, int, double*, int);
void refshim_strsm(enum CBLAS_ORDER, enum CBLAS_SIDE, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE,
                   enum CBLAS_DIAG, int, int, float, const float*, int, float*, int);
void refshim_dtrsv(enum CBLAS_ORDER, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE, enum CBLAS_DIAG,
                   int, const double*, int, double*, int);
void refshim_strsv(enum CBLAS_ORDER, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE, enum CBLAS_DIAG,
                   int, const float*, int, float*, int);
void refshim_dgemv(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, int, int, double, const double*, int,
                   const double*, int, double, double*, int);
void refshim_sgemv(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, int, int, float, const float*, int,
                   const float*, int, float, float*, int);
void refshim_dsyrk(enum CBLAS_ORDER, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE, int, int, double,
                   const double*, int, double, double*, int);
void refshim_ssyrk(enum CBLAS_ORDER, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE, int, int, float,
                   const float*, int, float, float*, int);
int  refshim_idamax(int, const double*, int);
int  refshim_isamax(int, const float*, int);
void refshim_dscal(int, double, double*, int);
void refshim_sscal(int, float, float*, int);
void refshim_dswap(int, double*, int, double*, int);
void refshim_sswap(int, float*, int, float*, int);

#if defined(DREAL)
   #define cblas_gemm refshim_dgemm
   #define cblas_trsm refshim_dtrsm
   #define cblas_syrk refshim_dsyrk
   #define cblas_trsv refshim_dtrsv
   #define cblas_gemv refshim_dgemv
   #define cblas_iamax refshim_idamax
   #define cblas_scal refshim_dscal
   #define cblas_swap refshim_dswap
#else
   #define cblas_gemm refshim_sgemm
   #define cblas_trsm refshim_strsm
   #define cblas_syrk refshim_ssyrk
   #define cblas_trsv refshim_strsv
   #define cblas_gemv refshim_sgemv
   #define cblas_iamax refshim_isamax
   #define cblas_scal refshim_sscal
   #define cblas_swap refshim_sswap
#endif
#endif
