#!/bin/sh
# Test infrastructure only: builds the reference Quanty CPU binary (unmodified sources,
# compiled where they lie) into oracle/_ref/, to generate golden fixtures and to check the
# oracle restatement against the reference itself.  Nothing in the product links or runs it.
#
# Recipe: the reference is one translation unit (LuaInterface/main.cpp includes every .cpp).
# It needs an LP64 BLAS/LAPACK; the one present in this image is scipy's bundled OpenBLAS,
# whose Fortran symbols carry a "scipy_" prefix, so a generated header maps the plain
# names onto the prefixed ones.  A second force-included header pins srand() so the
# reference's rand()-based starting vectors are reproducible.
#
# usage: oracle/build_ref.sh [reference-dir]      (default: /root/reference)
set -e
REF=${1:-${QUANTY_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT"
[ -f "$REF/LuaInterface/main.cpp" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
OB=$(python3 - <<'PY'
import glob, os, scipy
d = os.path.dirname(scipy.__file__) + ".libs"
c = [p for p in glob.glob(os.path.join(d, "libscipy_openblas*.so")) if "64_" not in os.path.basename(p)]
print(c[0] if c else "")
PY
)
[ -n "$OB" ] || { echo "no LP64 scipy OpenBLAS found" >&2; exit 1; }
nm -D --defined-only "$OB" | awk '$3 ~ /^scipy_/ { n = substr($3, 7); print "#define " n " " $3 }' > "$OUT/blas_names.h"
cat > "$OUT/pin_seed.h" <<'H'
#include <stdlib.h>
#define srand(x) srand(12345u)
H
ln -sf "$OB" "$OUT/libscipyob.so"
g++ "$REF/LuaInterface/main.cpp" -include "$OUT/blas_names.h" -include "$OUT/pin_seed.h" \
    -D LUA_USE_LINUX -DBLASunderscore -O2 -fopenmp -w \
    -L"$OUT" -lscipyob -Wl,-rpath,"$(dirname "$OB")" -o "$OUT/Quanty"
echo "built $OUT/Quanty"
