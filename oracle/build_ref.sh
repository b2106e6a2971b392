#!/bin/sh
# Test infrastructure only: builds the UNMODIFIED reference `smartpca`, `smartrel` and `convertf` (EIGENSOFT 8.0.0,
# DReichLab/EIG) from its own C sources where they lie, into oracle/_ref/ (git-ignored).
# The result is used to pin the oracle restatement and to generate the golden fixtures
# under tests/golden/.  Nothing of the product links or runs it.
#
# Recipe (the reference's own Makefile needs system OpenBLAS + GSL, absent here):
#   * gcc -O2 -fcommon: globals are defined in headers (include/globals.h:4-5).
#   * LAPACK symbols (dspev_, dpotrf_, ...) are forwarded to the scipy-bundled OpenBLAS,
#     which exports them with a `scipy_` prefix (ref_lapack_shim.c).
#   * fastmode (src/ksrc/kjg_fpca.c, kjg_gsl.c) is compiled against oracle/gsl_shim: the GSL
#     API subset it uses (views, gsl_blas_dgemm over CBLAS, GSL's default mt19937) written
#     from GSL's documentation, and LAPACKE from the same scipy-bundled OpenBLAS.
#   * fprintf is wrapped (-Wl,--wrap=fprintf, ref_fullprec.c): unchanged output unless
#     EIG_REF_FULLPREC=1, in which case the .eval/.evec number formats print %.17g so that
#     1e-10 parity can be checked; smartrel also wraps printf (its relatedness scores).  No reference source is modified or copied.
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
# the reference checkout: first argument, else $EIG_REFERENCE_DIR, else a sibling checkout
# named "reference" next to this repository
REF=${1:-${EIG_REFERENCE_DIR:-$HERE/../../reference}}
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "build_ref.sh: reference sources not present ($REF); nothing to build" >&2
  exit 0
fi
OPENBLAS=$(python3 - <<'EOF'
import glob, os, scipy
d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
libs = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
print(libs[0] if libs else "")
EOF
)
if [ -z "$OPENBLAS" ]; then
  echo "build_ref.sh: scipy-bundled OpenBLAS not found" >&2
  exit 1
fi
mkdir -p "$OUT/obj"
CFLAGS="-O2 -fcommon -w -U_FORTIFY_SOURCE -D_FORTIFY_SOURCE=0 -fno-builtin-fprintf -I$REF/include"
SRCS="$REF/src/nicksrc/gauss.c $REF/src/nicksrc/gds.c $REF/src/nicksrc/getpars.c
      $REF/src/nicksrc/linsubs.c $REF/src/nicksrc/sortit.c $REF/src/nicksrc/statsubs.c
      $REF/src/nicksrc/strsubs.c $REF/src/nicksrc/vsubs.c $REF/src/nicksrc/xsearch.c
      $REF/src/eigensrc/smartpca.c $REF/src/eigensrc/eigsubs.c $REF/src/eigensrc/exclude.c
      $REF/src/eigensrc/smartsubs.c $REF/src/eigensrc/eigx.c
      $REF/src/mcio.c $REF/src/qpsubs.c $REF/src/admutils.c $REF/src/egsubs.c
      $REF/src/regsubs.c $REF/src/gval.c $REF/src/twsubs.c"
OBJS=""
pids=""
for s in $SRCS; do
  o="$OUT/obj/$(basename "$(dirname "$s")")_$(basename "$s" .c).o"
  gcc $CFLAGS -c "$s" -o "$o" &
  pids="$pids $!"
  OBJS="$OBJS $o"
done
for p in $pids; do wait "$p"; done
gcc -O2 -c "$HERE/ref_lapack_shim.c" -o "$OUT/obj/ref_lapack_shim.o"
gcc -O2 -c "$HERE/ref_fullprec.c" -o "$OUT/obj/ref_fullprec.o"
gcc -O2 -I"$HERE/gsl_shim" -c "$HERE/gsl_shim/gsl_shim.c" -o "$OUT/obj/gsl_shim.o"
for k in kjg_fpca kjg_gsl; do
  gcc $CFLAGS -I"$HERE/gsl_shim" -c "$REF/src/ksrc/$k.c" -o "$OUT/obj/ksrc_$k.o"
done
gcc -o "$OUT/smartpca.new" $OBJS "$OUT/obj/ref_lapack_shim.o" "$OUT/obj/ref_fullprec.o" \
    "$OUT/obj/ksrc_kjg_fpca.o" "$OUT/obj/ksrc_kjg_gsl.o" "$OUT/obj/gsl_shim.o" -Wl,--wrap=fprintf \
    "$OPENBLAS" -Wl,-rpath,"$(dirname "$OPENBLAS")" -lm -lpthread
mv -f "$OUT/smartpca.new" "$OUT/smartpca"
echo "built $OUT/smartpca"
# smartrel (src/Makefile: smartrel.o twsubs mcio qpsubs admutils egsubs regsubs eigsubs eigx
# smartsubs + libnick) from the same objects
gcc $CFLAGS -fno-builtin-printf -c "$REF/src/eigensrc/smartrel.c" -o "$OUT/obj/eigensrc_smartrel.o"
RELOBJS=""
for o in $OBJS; do
  case "$o" in
    *eigensrc_smartpca.o|*eigensrc_exclude.o|*_gval.o) ;;
    *) RELOBJS="$RELOBJS $o" ;;
  esac
done
gcc -o "$OUT/smartrel" "$OUT/obj/eigensrc_smartrel.o" $RELOBJS "$OUT/obj/ref_lapack_shim.o" \
    "$OUT/obj/ref_fullprec.o" -Wl,--wrap=fprintf -Wl,--wrap=printf \
    "$OPENBLAS" -Wl,-rpath,"$(dirname "$OPENBLAS")" -lm -lpthread
echo "built $OUT/smartrel"
# convertf (src/Makefile: convertf.o mcio egsubs admutils h2d eigensrc/exclude + libnick)
gcc $CFLAGS -c "$REF/src/convertf.c" -o "$OUT/obj/convertf.o"
gcc $CFLAGS -c "$REF/src/h2d.c" -o "$OUT/obj/h2d.o"
CVOBJS=""
for o in $OBJS; do
  case "$o" in
    *nicksrc_*|*_mcio.o|*_egsubs.o|*_admutils.o|*eigensrc_exclude.o) CVOBJS="$CVOBJS $o" ;;
  esac
done
gcc -o "$OUT/convertf" "$OUT/obj/convertf.o" "$OUT/obj/h2d.o" $CVOBJS "$OUT/obj/ref_lapack_shim.o" \
    "$OPENBLAS" -Wl,-rpath,"$(dirname "$OPENBLAS")" -lm -lpthread
echo "built $OUT/convertf"
