/*
 * atlas_oracle.c -- CPU restatement of ATLAS 3.11.42's Level-3 / LU path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for math-atlas_gb300.  Only tests/,
 * the smoke test and bench.py's CPU-baseline leg use it.  Built with
 * -ffp-contract=off so that x86-64 and aarch64 hosts produce identical bits.
 *
 * Each routine cites the reference basefile it restates.  The
 * double/float bodies are in oracle_tmpl.inc.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "atlas_oracle.h"

enum { CblasRowMajor = 101, CblasColMajor = 102 };
enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum { CblasUpper = 121, CblasLower = 122 };
enum { CblasNonUnit = 131, CblasUnit = 132 };
enum { CblasLeft = 141, CblasRight = 142 };

#define ORA_FILLCONST (-2560000000.0)   /* atlas-tst.base:2951 */

static long ora_l1c_elts = 4096;
static int  ora_lcmmn = 0;

void ora_set_lu_params(long l1c_elts, int lcmmn)
{
   ora_l1c_elts = l1c_elts;
   ora_lcmmn = lcmmn;
}

int ora_set_threads(int n)
{
#ifdef _OPENMP
   if (n > 0) omp_set_num_threads(n);
   return omp_get_max_threads();
#else
   (void)n;
   return 1;
#endif
}

int ora_get_threads(void)
{
#ifdef _OPENMP
   return omp_get_max_threads();
#else
   return 1;
#endif
}

/* ----------------------------------------------------------------------- */
/* The test library's portable LCG (AtlasBase/Clint/atlas-tst.base:5353-    */
/* 5560): a 31-bit state kept as two ints (low 16 bits, high 15 bits),      */
/* x <- x*a + c mod 2^31 with a = 16838*2^16 + 20077, c = 12345.  The seed  */
/* enters as {seed, seed>>16} without masking the low word, exactly as the  */
/* reference's ATL_srand does; the arithmetic wraps in 32 bits as the       */
/* reference's int arithmetic does on two's-complement hardware.            */
/* ----------------------------------------------------------------------- */
static int rs_irand[2], rs_ias[2], rs_ics[2];

static int wmul(int a, int b) { return (int)((unsigned)a * (unsigned)b); }
static int wadd(int a, int b) { return (int)((unsigned)a + (unsigned)b); }

static void rs_ladd(const int *J, const int *K, int *I)
{
   int t0 = wadd(K[0], J[0]), t1;
   t1 = t0 >> 16;
   I[0] = t0 - (t1 << 16);
   t0 = wadd(wadd(t1, K[1]), J[1]);
   I[1] = t0 - ((t0 >> 15) << 15);
}

static void rs_lmul(const int *K, const int *J, int *I)
{
   const int p30 = 1 << 30;
   int kt, lt;
   kt = wmul(K[0], J[0]);
   if (kt < 0) kt = (kt + p30) + p30;
   I[0] = kt - ((kt >> 16) << 16);
   lt = wadd(wmul(K[0], J[1]), wmul(K[1], J[0]));
   if (lt < 0) lt = (lt + p30) + p30;
   kt = wadd(kt >> 16, lt);
   if (kt < 0) kt = (kt + p30) + p30;
   I[1] = kt - ((kt >> 15) << 15);
}

void ora_srand(int seed)
{
   const int mult[2] = {20077, 16838}, iadd[2] = {12345, 0};
   int jseed[2], j[2];
   jseed[0] = seed;
   jseed[1] = seed >> 16;
   rs_lmul(jseed, mult, j);
   rs_ladd(j, iadd, rs_irand);
   rs_ias[0] = mult[0]; rs_ias[1] = mult[1];
   rs_ics[0] = iadd[0]; rs_ics[1] = iadd[1];
}

int ora_rand(void)
{
   int cur[2], j[2];
   cur[0] = rs_irand[0]; cur[1] = rs_irand[1];
   rs_lmul(rs_irand, rs_ias, j);
   rs_ladd(j, rs_ics, rs_irand);
   return cur[0] + (cur[1] << 16);
}

/* ATL_epsilon (atlas-tst.base:3052): halve until 1+f rounds to 1 */
double ora_depsilon(void)
{
   double eps;
   volatile double maxval, f1 = 0.5;
   do { eps = f1; f1 *= 0.5; maxval = 1.0 + f1; } while (maxval != 1.0);
   return eps;
}

float ora_sepsilon(void)
{
   float eps;
   volatile float maxval, f1 = 0.5f;
   do { eps = f1; f1 *= 0.5f; maxval = 1.0f + f1; } while (maxval != 1.0f);
   return eps;
}

void ora_dgefillgap(int M, int N, double *A, int lda)
{
   int i, j;
   for (j = 0; j < N; j++)
      for (i = M; i < lda; i++) A[i + (size_t)j*lda] = ORA_FILLCONST;
}

int ora_dgechkgap(int M, int N, const double *A, int lda)
{
   int i, j, bad = 0;
   for (j = 0; j < N; j++)
      for (i = M; i < lda; i++)
         if (A[i + (size_t)j*lda] != ORA_FILLCONST) bad++;
   return bad;
}

/* ---- instantiate the type-generic body ---------------------------------- */
#define T double
#define P(x) ora_d##x
#define Q(x) d_##x
#define SAFMIN_T DBL_MIN
#define EPS_T ora_depsilon()
#include "oracle_tmpl.inc"
#undef T
#undef P
#undef Q
#undef SAFMIN_T
#undef EPS_T
#undef OPA
#undef OPT
#undef OPBLK
#undef ORA_MC
#undef ORA_NC
#undef ORA_KC
#undef ORA_TRB

#define T float
#define P(x) ora_s##x
#define Q(x) s_##x
#define SAFMIN_T FLT_MIN
#define EPS_T ora_sepsilon()
#include "oracle_tmpl.inc"
#undef T
#undef P
#undef Q
#undef SAFMIN_T
#undef EPS_T

int ora_idamax(int N, const double *X, int incX) { return d_iamax(N, X, incX); }
int ora_isamax(int N, const float *X, int incX) { return s_iamax(N, X, incX); }

int ora_dgesv(int Order, int N, int NRHS, double *A, int lda, int *ipiv,
              double *B, int ldb)
{
   int ierr = ora_dgetrf(Order, N, N, A, lda, ipiv);
   if (!ierr) ora_dgetrs(Order, CblasNoTrans, N, NRHS, A, lda, ipiv, B, ldb);
   return ierr;
}

/* gemmtst residual (AtlasBase/Antoine/atlbinblas.base:11853-11930) */
double ora_dgemm_resid(int TA, int TB, int M, int N, int K, double alpha,
                       const double *A, int lda, const double *B, int ldb,
                       double beta, const double *Cin, const double *Ctest,
                       const double *Ctrust, int ldc)
{
   const int mA = (TA == CblasNoTrans) ? M : K, nA = (TA == CblasNoTrans) ? K : M;
   const int mB = (TB == CblasNoTrans) ? K : N, nB = (TB == CblasNoTrans) ? N : K;
   double nA1, nB1, nC1, nD, mx;
   if (M == 0 || N == 0) return 0.0;
   nC1 = ora_dgenrm1(M, N, Cin, ldc);
   if (fabs(beta) > 1.0) nC1 *= fabs(beta);
   if (nC1 == 0.0) nC1 = 1.0;
   nA1 = ora_dgenrm1(mA, nA, A, lda);
   if (fabs(alpha) > 1.0) nA1 *= fabs(alpha);
   if (nA1 == 0.0) nA1 = 1.0;
   nB1 = ora_dgenrm1(mB, nB, B, ldb);
   if (nB1 == 0.0) nB1 = 1.0;
   nD = ora_dgediffnrm1(M, N, Ctest, ldc, Ctrust, ldc);
   mx = (M > N) ? M : N;
   if (K > mx) mx = K;
   return nD / ((nA1 > 1.0 ? nA1 : 1.0) * (nB1 > 1.0 ? nB1 : 1.0) *
                (nC1 > 1.0 ? nC1 : 1.0) * ora_depsilon() * mx);
}

/* slvtst residual (AtlasBase/Clint/atlas-tlp.base:574-600) */
double ora_dslv_resid(int N, int NRHS, const double *A, int lda,
                      const double *X, int ldx, const double *Xc, int ldxc)
{
   double nA = ora_dgenrm1(N, N, A, lda), nd = 0.0, nx = 0.0;
   int i, j;
   for (j = 0; j < NRHS; j++)
      for (i = 0; i < N; i++)
      {
         const double d = fabs(X[i + (size_t)j*ldx] - Xc[i + (size_t)j*ldxc]);
         const double x = fabs(Xc[i + (size_t)j*ldxc]);
         if (d > nd) nd = d;
         if (x > nx) nx = x;
      }
   if (nA == 0.0) nA = 1.0;
   if (nx == 0.0) nx = 1.0;
   return nd / ((double)N * ora_depsilon() * nA * nx);
}

/* ----------------------------------------------------------------------- */
/* Double-double arithmetic from the published error-free transformations:  */
/* Knuth's TwoSum and Dekker's TwoProduct with Veltkamp splitting (Dekker,  */
/* "A floating-point technique for extending the available precision",     */
/* Numer. Math. 18, 1971).  No fused multiply-add is assumed.               */
/* ----------------------------------------------------------------------- */
static void two_sum(double a, double b, double *s, double *e)
{
   volatile double x = a + b;
   volatile double bv = x - a;
   volatile double av = x - bv;
   *s = x;
   *e = (a - av) + (b - bv);
}

static void split53(double a, double *hi, double *lo)
{
   volatile double c = 134217729.0 * a;   /* 2^27 + 1 */
   volatile double h = c - (c - a);
   *hi = h;
   *lo = a - h;
}

static void two_prod(double a, double b, double *p, double *e)
{
   double ah, al, bh, bl;
   volatile double x = a * b;
   split53(a, &ah, &al);
   split53(b, &bh, &bl);
   *p = x;
   *e = ((ah*bh - x) + ah*bl + al*bh) + al*bl;
}

static void dd_add(double *hi, double *lo, double b, double bl)
{
   double s, e, t;
   two_sum(*hi, b, &s, &e);
   e += *lo + bl;
   t = s + e;
   *lo = e - (t - s);
   *hi = t;
}

void ora_dgemm_dd_samples(int TA, int TB, int M, int N, int K,
                          const double *A, int lda, const double *B, int ldb,
                          int nsamp, const int *ii, const int *jj,
                          double *hi, double *lo)
{
   int s;
   (void)M; (void)N;
   #pragma omp parallel for schedule(dynamic, 4)
   for (s = 0; s < nsamp; s++)
   {
      double h = 0.0, l = 0.0;
      int k;
      for (k = 0; k < K; k++)
      {
         const double a = (TA == CblasNoTrans) ? A[ii[s] + (size_t)k*lda]
                                               : A[k + (size_t)ii[s]*lda];
         const double b = (TB == CblasNoTrans) ? B[k + (size_t)jj[s]*ldb]
                                               : B[jj[s] + (size_t)k*ldb];
         double p, e;
         two_prod(a, b, &p, &e);
         dd_add(&h, &l, p, e);
      }
      hi[s] = h;
      lo[s] = l;
   }
}

double ora_dbackward_error(int N, const double *A, int lda, const double *x,
                           const double *b)
{
   double rmax = 0.0, amax = 0.0, xmax = 0.0, bmax = 0.0;
   int i;
   #pragma omp parallel for reduction(max:rmax, amax)
   for (i = 0; i < N; i++)
   {
      double h = b[i], l = 0.0, arow = 0.0;
      int k;
      for (k = 0; k < N; k++)
      {
         double p, e;
         const double a = A[i + (size_t)k*lda];
         two_prod(-a, x[k], &p, &e);
         dd_add(&h, &l, p, e);
         arow += fabs(a);
      }
      if (fabs(h + l) > rmax) rmax = fabs(h + l);
      if (arow > amax) amax = arow;
   }
   for (i = 0; i < N; i++)
   {
      if (fabs(x[i]) > xmax) xmax = fabs(x[i]);
      if (fabs(b[i]) > bmax) bmax = fabs(b[i]);
   }
   return rmax / (amax * xmax + bmax);
}
