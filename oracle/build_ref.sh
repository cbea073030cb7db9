#!/bin/sh
# Compiles the reference's own CPU k-means (KmeansNaive, KmeansInitializer)
# unchanged from the reference tree into oracle/_ref/libckm_ref_naive.so.
# Flags follow the reference's CMakeLists.txt (-std=c++14 -O3
# -ffp-contract=fast), without -march=native so the result is portable.
# Usage: oracle/build_ref.sh [REFERENCE_DIR]   (default /root/reference)
set -e
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$REF/kmeans_naive.cpp" ]; then
    echo "reference tree not found at $REF; skipping oracle/_ref" >&2
    exit 0
fi
EXTRA=""
case "$(uname -m)" in
    x86_64) EXTRA="-mfma" ;;   # the reference's -march=native implies FMA here
esac
mkdir -p "$HERE/_ref"
g++ -std=c++14 -O3 -ffp-contract=fast $EXTRA -fPIC -shared \
    -I"$HERE/ref_stub" -I"$REF" \
    "$HERE/ref_naive_shim.cpp" -o "$HERE/_ref/libckm_ref_naive.so"
echo "built $HERE/_ref/libckm_ref_naive.so"
