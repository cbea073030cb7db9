#!/bin/sh
# Compiles the reference's own CPU k-means (KmeansNaive, KmeansInitializer)
# unchanged into oracle/_ref/libckm_ref_naive.so.
#
# Flags follow the reference's CMakeLists.txt (-std=c++14 -O3
# -ffp-contract=fast), without -march=native so the result is portable.
#
# Usage: oracle/build_ref.sh [REFERENCE_DIR]
#   REFERENCE_DIR defaults to $CKM_REFERENCE_DIR, else /root/reference.
#
# The GPU machines have no reference tree and keep no x86 binary built here.
# So, when the tree is present, the handful of reference files the shim
# includes (listed by the compiler's own dependency scan) are staged unchanged
# under oracle/_ref/src/ -- a git-ignored build folder, never committed -- and
# the library is compiled from there.  A machine without the tree compiles
# the staged files it received; with neither, the step is skipped.
set -e
REF="${1:-${CKM_REFERENCE_DIR:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
STAGE="$HERE/_ref/src"
if [ -f "$REF/kmeans_naive.cpp" ]; then
    REF="$(cd "$REF" && pwd)"
    mkdir -p "$STAGE"
    for f in $(g++ -std=c++14 -MM -I"$HERE/ref_stub" -I"$REF" "$HERE/ref_naive_shim.cpp" \
               | tr -d '\\' | tr ' ' '\n' | grep "^$REF/"); do
        rel="${f#$REF/}"
        mkdir -p "$STAGE/$(dirname "$rel")"
        cp -p "$f" "$STAGE/$rel"
    done
elif [ ! -f "$STAGE/kmeans_naive.cpp" ]; then
    echo "reference tree not found at $REF and no staged copy; skipping oracle/_ref" >&2
    exit 0
fi
EXTRA=""
case "$(uname -m)" in
    x86_64) EXTRA="-mfma" ;;   # the reference's -march=native implies FMA here
esac
g++ -std=c++14 -O3 -ffp-contract=fast $EXTRA -fPIC -shared \
    -I"$HERE/ref_stub" -I"$STAGE" \
    "$HERE/ref_naive_shim.cpp" -o "$HERE/_ref/libckm_ref_naive.so"
echo "built $HERE/_ref/libckm_ref_naive.so"
