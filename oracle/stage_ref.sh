#!/bin/bash
# Test and measurement infrastructure only: copies the reference's C/C++ sources (and the
# reference test scripts the drop-in check runs) into baseline/_ref/, the git-ignored folder the
# reference is installed into, so that machines without the reference tree (the GPU host) can
# build the reference's own binaries there (oracle/build_ref.sh baseline/_ref).  Nothing is
# copied into tracked files.
#
# usage: oracle/stage_ref.sh [reference-dir]      (default: $QUANTY_REFERENCE, else /root/reference)
set -e
REF=${1:-${QUANTY_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
DEST="$HERE/../baseline/_ref"
[ -f "$REF/LuaInterface/main.cpp" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
mkdir -p "$DEST"
cd "$REF"
find . -type f \( -name "*.cpp" -o -name "*.c" -o -name "*.h" -o -name "*.hpp" -o -name "*.inc" -o -name "*.cc" \) \
    -not -path "./TestScripts/*" -not -path "./Debug examples/*" -not -path "./.git/*" -print0 |
    xargs -0 cp --parents -t "$DEST"
mkdir -p "$DEST/TestScripts"
for t in CreateSpectra Eigensystem CreateResonantSpectra; do cp "TestScripts/$t.Quanty" "$DEST/TestScripts/"; done
echo "staged $(cd "$DEST" && pwd)"
