#!/usr/bin/env bash
# Builds the reference's own per-pixel stage bodies for the host CPU into
# oracle/_ref/ (test infrastructure: pins the C restatement and generates the
# golden fixtures). Reads the reference checkout in place; the one patched
# file (the Y threshold macro for the Y=48 variant) is written to a temporary
# directory outside the repository and deleted afterwards.
#
# usage: oracle/build_ref.sh [REFERENCE_DIR]   (default /root/reference)
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/graph_functions.cu" ]; then
    echo "build_ref: no reference checkout at $REF; skipped" >&2
    exit 0
fi
mkdir -p "$OUT"
TMP="$(mktemp -d)"
trap 'rm -rf "$TMP"' EXIT
# Y=48 variant: the reference keeps the original threshold commented out
# (graph_functions.cu:15) and builds with 5 (graph_functions.cu:17).
sed 's/^#define trY 0x00050000/#define trY 0x00300000/' "$REF/graph_functions.cu" > "$TMP/graph_functions.cu"
grep -q '^#define trY 0x00300000' "$TMP/graph_functions.cu"
FLAGS="-O2 -std=c++14 -fPIC -shared -w -ffp-contract=off"
g++ $FLAGS -I"$REF" "$HERE/ref_driver.cpp" -o "$OUT/libdepix_ref5.so" &
g++ $FLAGS -I"$TMP" -I"$REF" "$HERE/ref_driver.cpp" -o "$OUT/libdepix_ref48.so" &
wait
echo "build_ref: built $OUT/libdepix_ref5.so $OUT/libdepix_ref48.so"
