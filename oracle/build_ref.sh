#!/bin/bash
# Test and measurement infrastructure only: builds the reference's own CPU programs from its
# unmodified sources, compiled where they lie, into oracle/_ref/.  Nothing in the product links
# or runs them.
#   quanty  the reference binary (LuaInterface/main.cpp): golden fixtures, oracle pins
#   hpsi    oracle/ref_hpsi.cpp around the reference's translation unit: the reference's own
#           fixed-basis H*psi timed on a given basis (the CPU arm of bench.py) and its output
#   headers only the generated headers (BLAS name map, seed pin) other builds reuse
#
# Recipe: the reference is one translation unit (LuaInterface/main.cpp includes every .cpp).
# It needs an LP64 BLAS/LAPACK; the one present on these machines is scipy's bundled OpenBLAS,
# whose Fortran symbols carry a "scipy_" prefix, so a generated header maps the plain names
# onto the prefixed ones.  A second force-included header pins srand() so the reference's
# rand()-based starting vectors are reproducible.
#
# usage: oracle/build_ref.sh [reference-dir] [quanty|hpsi ...]
#        reference-dir defaults to $QUANTY_REFERENCE, else /root/reference; the targets to quanty
set -e
REF=${1:-${QUANTY_REFERENCE:-/root/reference}}
shift || true
TARGETS=${*:-quanty}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT"
[ -f "$REF/LuaInterface/main.cpp" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
REF=$(cd "$REF" && pwd)
OB=$(python3 - <<'PY'
import glob, os, scipy
d = os.path.dirname(scipy.__file__) + ".libs"
c = [p for p in glob.glob(os.path.join(d, "libscipy_openblas*.so")) if "64_" not in os.path.basename(p)]
print(c[0] if c else "")
PY
)
[ -n "$OB" ] || { echo "no LP64 scipy OpenBLAS found" >&2; exit 1; }
# written to temporary names and moved into place, so builds running side by side read whole files
nm -D --defined-only "$OB" | awk '$3 ~ /^scipy_/ { n = substr($3, 7); print "#define " n " " $3 }' > "$OUT/blas_names.h.$$"
mv -f "$OUT/blas_names.h.$$" "$OUT/blas_names.h"
printf '#include <stdlib.h>\n#define srand(x) srand(12345u)\n' > "$OUT/pin_seed.h.$$"
mv -f "$OUT/pin_seed.h.$$" "$OUT/pin_seed.h"
ln -sfn "$OB" "$OUT/libscipyob.so.$$" && mv -fT "$OUT/libscipyob.so.$$" "$OUT/libscipyob.so"
FLAGS=(-include "$OUT/blas_names.h" -include "$OUT/pin_seed.h" -D LUA_USE_LINUX -DBLASunderscore -O2 -fopenmp -w
       -L"$OUT" -lscipyob -Wl,-rpath,"$(dirname "$OB")")
for t in $TARGETS; do
  case $t in
    quanty) g++ "$REF/LuaInterface/main.cpp" "${FLAGS[@]}" -o "$OUT/Quanty" & ;;
    hpsi) g++ "$HERE/ref_hpsi.cpp" -I"$REF" "${FLAGS[@]}" -o "$OUT/ref_hpsi" & ;;
    headers) ;;  # only the BLAS name map and the seed pin (for builds made elsewhere)
    *) echo "unknown target $t" >&2; exit 2 ;;
  esac
done
fail=0
for job in $(jobs -p); do wait "$job" || fail=1; done
[ $fail = 0 ] || { echo "reference build failed" >&2; exit 1; }
echo "built $TARGETS in $OUT"
