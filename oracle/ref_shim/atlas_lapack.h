/* LAPACK-layer names used by the extracted routines.  TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_LAPACK_H
#define REFSHIM_LAPACK_H
#include "atlas_misc.h"
#define ATL_getrfC Mjoin(PATL,getrfC)
#define ATL_getrfR Mjoin(PATL,getrfR)
#define ATL_getrs  Mjoin(PATL,getrs)
#define ATL_laswp  Mjoin(PATL,laswp)
int  ATL_dgetrfC(const int, const int, double*, const int, int*);
int  ATL_sgetrfC(const int, const int, float*, const int, int*);
int  ATL_dgetrfR(const int, const int, double*, const int, int*);
int  ATL_sgetrfR(const int, const int, float*, const int, int*);
int  ATL_dgetf2(const int, const int, double*, const int, int*);
int  ATL_sgetf2(const int, const int, float*, const int, int*);
void ATL_dlaswp(const int, double*, const int, const int, const int, const int*, const int);
void ATL_slaswp(const int, float*, const int, const int, const int, const int*, const int);
void ATL_dgetrs(const enum CBLAS_ORDER, const enum CBLAS_TRANSPOSE, const int, const int,
                const double*, const int, const int*, double*, const int);
void ATL_sgetrs(const enum CBLAS_ORDER, const enum CBLAS_TRANSPOSE, const int, const int,
                const float*, const int, const int*, float*, const int);
#define ATL_potrfU Mjoin(PATL,potrfU)
#define ATL_potrfL Mjoin(PATL,potrfL)
#define ATL_potrf  Mjoin(PATL,potrf)
#define ATL_potrs  Mjoin(PATL,potrs)
int  ATL_dpotrfU(const int, double*, const int);
int  ATL_spotrfU(const int, float*, const int);
int  ATL_dpotrfL(const int, double*, const int);
int  ATL_spotrfL(const int, float*, const int);
int  ATL_dpotrf(const enum ATLAS_ORDER, const enum ATLAS_UPLO, const int, double*, const int);
int  ATL_spotrf(const enum ATLAS_ORDER, const enum ATLAS_UPLO, const int, float*, const int);
void ATL_dpotrs(const enum CBLAS_ORDER, const enum CBLAS_UPLO, const int, const int, const double*,
                const int, double*, const int);
void ATL_spotrs(const enum CBLAS_ORDER, const enum CBLAS_UPLO, const int, const int, const float*,
                const int, float*, const int);
#define ATL_trtri  Mjoin(PATL,trtri)
#define ATL_trtriCU Mjoin(PATL,trtriCU)
#define ATL_trtriCL Mjoin(PATL,trtriCL)
#define ATL_trtriRU Mjoin(PATL,trtriRU)
#define ATL_trtriRL Mjoin(PATL,trtriRL)
#define ATL_getri  Mjoin(PATL,getri)
#define ATL_getriC Mjoin(PATL,getriC)
#define ATL_getriR Mjoin(PATL,getriR)
int ATL_dtrtri(const enum ATLAS_ORDER, const enum ATLAS_UPLO, const enum ATLAS_DIAG, const int,
               double*, const int);
int ATL_strtri(const enum ATLAS_ORDER, const enum ATLAS_UPLO, const enum ATLAS_DIAG, const int,
               float*, const int);
int ATL_dtrtriCU(const enum ATLAS_DIAG, const int, double*, const int);
int ATL_strtriCU(const enum ATLAS_DIAG, const int, float*, const int);
int ATL_dtrtriCL(const enum ATLAS_DIAG, const int, double*, const int);
int ATL_strtriCL(const enum ATLAS_DIAG, const int, float*, const int);
int ATL_dtrtriRU(const enum ATLAS_DIAG, const int, double*, const int);
int ATL_strtriRU(const enum ATLAS_DIAG, const int, float*, const int);
int ATL_dtrtriRL(const enum ATLAS_DIAG, const int, double*, const int);
int ATL_strtriRL(const enum ATLAS_DIAG, const int, float*, const int);
int ATL_dgetri(const enum CBLAS_ORDER, const int, double*, const int, const int*, double*, int*);
int ATL_sgetri(const enum CBLAS_ORDER, const int, float*, const int, const int*, float*, int*);
int ATL_dgetriC(const int, double*, const int, const int*, double*, const int);
int ATL_sgetriC(const int, float*, const int, const int*, float*, const int);
int ATL_dgetriR(const int, double*, const int, const int*, double*, const int);
int ATL_sgetriR(const int, float*, const int, const int*, float*, const int);
/* blocking factor of the tuned build; the stand-in lives in ref_glue.c */
int ATL_dlaGetB(int, int, int, int);
int ATL_slaGetB(int, int, int, int);
void ATL_dger(const int, const int, const double, const double*, const int, const double*,
              const int, double*, const int);
void ATL_sger(const int, const int, const float, const float*, const int, const float*,
              const int, float*, const int);
#endif
