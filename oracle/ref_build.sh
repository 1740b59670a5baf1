#!/bin/sh
# Builds the reference's own routines and tester programs from its basefiles,
# for pinning the oracle and checking the GPU library (TEST INFRASTRUCTURE
# ONLY).
#
# usage: sh oracle/ref_build.sh [REFERENCE_TREE]
#   REFERENCE_TREE (or $ATLAS_REFERENCE) is the ATLAS developer tree (the
#   directory holding extract.c and AtlasBase/).  Given one, the script
#   extracts the sources into oracle/_ref/src and compiles them; without one
#   it compiles what an earlier run extracted there (a copy of the repository
#   made after an extraction carries oracle/_ref/src with it).
#
#  1. compiles the reference's basefile extractor (extract.c) with gcc;
#  2. extracts, one routine per file, ATL_getrfC/getrfR/getf2/laswp/getrs and
#     ATL_potrfU/potrfL/potrf/potrs, ATL_trtri* and ATL_getri*
#     (AtlasBase/Clint/atlas-lp.base),
#     ATL_rand/gegen/epsilon (AtlasBase/Clint/atlas-tst.base), ATL_iamax
#     (AtlasBase/Clint/atlas-lvl1.base) and the C
#     reference BLAS they run on (gemm, trsm, trmm, syrk, gemv, trsv, ger, scal,
#     swap, iamax, plus symm, syr2k, asum, copy for the testers, from
#     AtlasBase/Antoine/atlrefblas.base);
#  3. compiles them, double and single precision, with the stand-in headers in
#     oracle/ref_shim/ into oracle/_ref/libatlref.so;
#  4. extracts the tester programs xdlutst (`lutst`,
#     AtlasBase/Clint/atlas-tlp.base, built with -DTimeC so it factors through
#     clapack_dgetrf) and xdl3blastst (`l3blastst`,
#     AtlasBase/Antoine/atlbinblas.base, built with -DUSE_L3_REFERENCE so the
#     trusted GEMM is the reference BLAS) with the test-library routines they
#     call (AtlasBase/Clint/atlas-tst.base, atlasBV.base, atlas-iaux.base,
#     atlas.base), and, when math-atlas_gb300/libatlas_gb300.so exists, links
#     them against it (oracle/ref_shim/tester_glue.c binds their internal names)
#     into oracle/_ref/xdlutst and oracle/_ref/xdl3blastst.
# Everything it writes goes to oracle/_ref/ (git-ignored).  The reference's own
# make system, configure step and tuned kernels are not used.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-$ATLAS_REFERENCE}
OUT=$HERE/_ref
SRC=$OUT/src
TST=$SRC/tst
CC=${CC:-gcc}
if [ -n "$REF" ]; then
   R=$REF/AtlasBase
   mkdir -p "$SRC" "$TST"
   $CC -ansi -O2 -w -o "$OUT/xextract" "$REF/extract.c"
   X="$OUT/xextract -langC -lnlen79 -Remtblank -def topd $R -def BASEdir $R/Antoine/ -def incd $R/Clint -def basd $R/Clint"
   cd "$SRC"
   $X -b $R/Clint/atlas.base -o atlas_enum.h rout=atlas_enum.h
   $X -b $R/Clint/atlas.base -o cblas.h rout=cblas.h
   for h in misc lvl3 level3 level1 level2 lvl2; do
      $X -b $R/Antoine/atlrefblas.base -o atlas_ref$h.h rout=atlas_ref$h.h type=none
   done
   RB="gemm gemmNN gemmNT gemmTN gemmTT trsm trmm ger scal swap syrk syrkLN syrkLT syrkUN syrkUT"
   RB="$RB gemv gemvN gemvT trsv asum copy symm syr2k"
   for s in L R; do for u in L U; do RB="$RB symm$s$u"; done; done
   for u in L U; do for t in N T; do RB="$RB syr2k$u$t"; done; done
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
   # tester programs and the test-library routines they call
   cd "$TST"
   $X -b $R/Clint/atlas-tlp.base -o lutst.c rout=lutst
   $X -b $R/Antoine/atlbinblas.base -o l3blastst.c rout=l3blastst type=dble
   for r in ATL_genrm1 ATL_gediffnrm1 ATL_synrm ATL_trnrm1 ATL_gecmpBV ATL_trcmpBV ATL_print2dBV; do
      $X -b $R/Clint/atlas-tst.base -o $r.c rout=$r
   done
   $X -b $R/Clint/atlasBV.base -o atlas_bitvec.h rout=atlas_bitvec.h
   for r in ATL_NewBV ATL_GetTotBitsBV ATL_SetBitBV ATL_FindFirstSetBitBV; do
      $X -b $R/Clint/atlasBV.base -o $r.c rout=$r
   done
   $X -b $R/Clint/atlas-iaux.base -o ATL_flushcache.c rout=ATL_flushcache
   $X -b $R/Clint/atlas.base -o time00.c rout=time00
fi
if [ ! -f "$SRC/ATL_getrfC.c" ]; then
   echo "ref_build.sh: no reference tree given and nothing extracted in $SRC" >&2
   exit 1
fi
cd "$SRC"
# objects compiled on an earlier machine are not reused (the copy may be on another architecture)
rm -f ./*.o "$TST"/*.o
CF="-O2 -fPIC -w -ffp-contract=off -fno-strict-aliasing -fwrapv -I$SRC -I$HERE/ref_shim"
OBJ=""
for f in ATL_dref*.c ATL_idrefamax.c; do $CC $CF -DDREAL -c $f -o ${f%.c}.o & OBJ="$OBJ ${f%.c}.o"; done
wait
for f in ATL_sref*.c ATL_isrefamax.c; do $CC $CF -DSREAL -c $f -o ${f%.c}.o & OBJ="$OBJ ${f%.c}.o"; done
wait
for f in ATL_getrfC ATL_getrfR ATL_getf2 ATL_laswp ATL_getrs ATL_potrfU ATL_potrfL ATL_potrf ATL_potrs \
         ATL_trtri ATL_trtriCU ATL_trtriCL ATL_trtriRU ATL_trtriRL ATL_getri ATL_getriC ATL_getriR \
         ATL_gegen ATL_epsilon ATL_iamax; do
   $CC $CF -DDREAL -c $f.c -o d_$f.o &
   $CC $CF -DSREAL -c $f.c -o s_$f.o &
   OBJ="$OBJ d_$f.o s_$f.o"
done
wait
$CC $CF -DDREAL -c ATL_rand.c -o ATL_rand.o
$CC $CF -c "$HERE/ref_shim/ref_glue.c" -o ref_glue.o
$CC -shared -o "$OUT/libatlref.so" $OBJ ATL_rand.o ref_glue.o -lm
echo "built $OUT/libatlref.so"

GB=$HERE/../math-atlas_gb300
if [ -f "$GB/libatlas_gb300.so" ] && [ -f "$TST/lutst.c" ]; then
   cd "$TST"
   # L2SIZE: the install-time cache size the testers flush with (4 MiB, lutst's default)
   TF="-O2 -Werror=implicit-function-declaration -Werror=implicit-int -ffp-contract=off -fno-strict-aliasing -fwrapv -DL2SIZE=4194304 -I$TST -I$HERE/ref_shim/tester -I$SRC -I$HERE/ref_shim"
   TOBJ=""
   for f in ATL_genrm1 ATL_gediffnrm1 ATL_synrm ATL_trnrm1 ATL_gecmpBV ATL_trcmpBV ATL_print2dBV ATL_flushcache \
            ATL_NewBV ATL_GetTotBitsBV ATL_SetBitBV ATL_FindFirstSetBitBV; do
      $CC $TF -DDREAL -c $f.c -o $f.o & TOBJ="$TOBJ $f.o"
   done
   $CC $TF -DWALL -c time00.c -o time00.o &
   $CC $TF -DDREAL -DTimeC -c lutst.c -o lutst.o &
   $CC $TF -DDREAL -DUSE_L3_REFERENCE -c l3blastst.c -o l3blastst.o &
   $CC $TF -c "$HERE/ref_shim/tester_glue.c" -o tester_glue.o &
   wait
   LINK="-L$OUT -latlref -L$GB -latlas_gb300 -Wl,-rpath,$OUT -Wl,-rpath,$GB -lm"
   $CC -o "$OUT/xdlutst" lutst.o $TOBJ time00.o tester_glue.o $LINK
   $CC -o "$OUT/xdl3blastst" l3blastst.o $TOBJ time00.o tester_glue.o $LINK
   echo "built $OUT/xdlutst $OUT/xdl3blastst"
fi
