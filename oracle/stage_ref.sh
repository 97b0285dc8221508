#!/bin/bash
# Test and measurement infrastructure only: copies the reference's source tree (and the
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
# everything the one translation unit includes (sources and headers of any extension, e.g.
# Simon/*.class) -- the whole tree except its test scripts, examples, documentation and history
find . -type f -not -path "./TestScripts/*" -not -path "./Debug examples/*" -not -path "./Doc/*" \
    -not -path "./Test/*" -not -path "./.git/*" -print0 | xargs -0 cp --parents -t "$DEST"
mkdir -p "$DEST/TestScripts"
for t in CreateSpectra Eigensystem CreateResonantSpectra; do cp "TestScripts/$t.Quanty" "$DEST/TestScripts/"; done
echo "staged $(cd "$DEST" && pwd)"
