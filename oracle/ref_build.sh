#!/bin/sh
# Builds the reference's own LU-path routines from its basefiles, for pinning
# the oracle (TEST INFRASTRUCTURE ONLY).
#
#  1. compiles the reference's basefile extractor (extract.c) with gcc;
#  2. extracts, one routine per file, ATL_getrfC/getrfR/getf2/laswp/getrs and
#     ATL_potrfU/potrfL/potrf/potrs, ATL_trtri* and ATL_getri*
#     (AtlasBase/Clint/atlas-lp.base),
#     ATL_rand/gegen/epsilon (AtlasBase/Clint/atlas-tst.base), ATL_iamax
#     (AtlasBase/Clint/atlas-lvl1.base) and the C
#     reference BLAS they run on (gemm, trsm, trmm, syrk, gemv, trsv, ger, scal,
#     swap, iamax from
#     AtlasBase/Antoine/atlrefblas.base);
#  3. compiles them, double and single precision, with the stand-in headers in
#     oracle/ref_shim/ into oracle/_ref/libatlref.so.
# Everything it writes goes to oracle/_ref/ (git-ignored).  The reference's own
# make system, configure step and tuned kernels are not used.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${ATLAS_REFERENCE:-/root/reference}
OUT=$HERE/_ref
SRC=$OUT/src
mkdir -p "$SRC"
R=$REF/AtlasBase
CC=${CC:-gcc}
$CC -ansi -O2 -w -o "$OUT/xextract" "$REF/extract.c"
X="$OUT/xextract -langC -lnlen79 -Remtblank -def topd $R -def BASEdir $R/Antoine/ -def incd $R/Clint -def basd $R/Clint"
cd "$SRC"
$X -b $R/Clint/atlas.base -o atlas_enum.h rout=atlas_enum.h
$X -b $R/Clint/atlas.base -o cblas.h rout=cblas.h
for h in misc lvl3 level3 level1 level2 lvl2; do
   $X -b $R/Antoine/atlrefblas.base -o atlas_ref$h.h rout=atlas_ref$h.h type=none
done
RB="gemm gemmNN gemmNT gemmTN gemmTT trsm trmm ger scal swap syrk syrkLN syrkLT syrkUN syrkUT"
RB="$RB gemv gemvN gemvT trsv"
for s in L R; do for u in L U; do for t in N T; do for d in N U; do RB="$RB trsm$s$u$t$d trmm$s$u$t$d"; done; done; done; done
for u in L U; do for t in N T; do for d in N U; do RB="$RB trsv$u$t$d"; done; done; done
for r in $RB; do
   $X -b $R/Antoine/atlrefblas.base -o ATL_dref$r.c rout=$r type=dble
   $X -b $R/Antoine/atlrefblas.base -o ATL_sref$r.c rout=$r type=real
done
$X -b $R/Antoine/atlrefblas.base -o ATL_idrefamax.c rout=amax type=dble
$X -b $R/Antoine/atlrefblas.base -o ATL_isrefamax.c rout=amax type=real
for r in ATL_getrfC ATL_getrfR ATL_getf2 ATL_laswp ATL_getrs ATL_potrfU ATL_potrfL ATL_potrf ATL_potrs \
         ATL_trtri ATL_trtriCU ATL_trtriCL ATL_trtriRU ATL_trtriRL ATL_getri ATL_getriC ATL_getriR; do
   $X -b $R/Clint/atlas-lp.base -o $r.c rout=$r 2>/dev/null
done
for r in ATL_rand ATL_gegen ATL_epsilon; do
   $X -b $R/Clint/atlas-tst.base -o $r.c rout=$r
done
$X -b $R/Clint/atlas-lvl1.base -o ATL_iamax.c rout=ATL_iamax
CF="-O2 -fPIC -w -ffp-contract=off -fno-strict-aliasing -fwrapv -I$SRC -I$HERE/ref_shim"
OBJ=""
for f in ATL_dref*.c ATL_idrefamax.c; do $CC $CF -DDREAL -c $f -o ${f%.c}.o; OBJ="$OBJ ${f%.c}.o"; done
for f in ATL_sref*.c ATL_isrefamax.c; do $CC $CF -DSREAL -c $f -o ${f%.c}.o; OBJ="$OBJ ${f%.c}.o"; done
for f in ATL_getrfC ATL_getrfR ATL_getf2 ATL_laswp ATL_getrs ATL_potrfU ATL_potrfL ATL_potrf ATL_potrs \
         ATL_trtri ATL_trtriCU ATL_trtriCL ATL_trtriRU ATL_trtriRL ATL_getri ATL_getriC ATL_getriR \
         ATL_gegen ATL_epsilon ATL_iamax; do
   $CC $CF -DDREAL -c $f.c -o d_$f.o
   $CC $CF -DSREAL -c $f.c -o s_$f.o
   OBJ="$OBJ d_$f.o s_$f.o"
done
$CC $CF -DDREAL -c ATL_rand.c -o ATL_rand.o
$CC $CF -c "$HERE/ref_shim/ref_glue.c" -o ref_glue.o
$CC -shared -o "$OUT/libatlref.so" $OBJ ATL_rand.o ref_glue.o -lm
echo "built $OUT/libatlref.so"
