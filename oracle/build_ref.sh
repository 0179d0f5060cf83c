#!/usr/bin/env bash
# Builds the reference's own per-pixel stage bodies into oracle/_ref/ (test
# infrastructure: the parity targets of the oracle and of the library, and the
# timed CPU baseline):
#   libdepix_ref{5,48}.so     host build (g++, IEEE, no contraction), ref_driver.cpp
#   libdepix_refgpu{5,48}.so  CUDA build for sm_103a with the reference's own
#                             device flags (depixel_gpu.pro:48), ref_gpu.cu
# 5 and 48 are the Y thresholds: the reference builds with 5
# (graph_functions.cu:17) and keeps the original 48 commented out
# (graph_functions.cu:15); the 48 variant is a copy with that one line changed.
#
# Sources: the reference's five stage files are copied into oracle/_ref/src
# (and the patched one into oracle/_ref/src48). That directory is git-ignored
# and never committed; it travels with the working tree to the machine that
# runs the GPU tests, where no reference checkout exists, so the same script
# rebuilds both variants there for that machine's CPU.
#
# usage: oracle/build_ref.sh [REFERENCE_DIR]
#   REFERENCE_DIR defaults to $DEPIX_REFERENCE_DIR, then /root/reference; when
#   it holds no checkout, the staged copy in oracle/_ref/src is used.
#   DEPIX_REF_NO_GPU=1 skips the CUDA build (no nvcc).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
SRC48="$OUT/src48"
REF="${1:-${DEPIX_REFERENCE_DIR:-/root/reference}}"
FILES="point.cu graph_functions.cu diagram_functions.cu subdivision_functions.cu triangulate_functions.cu"

mkdir -p "$OUT"
if [ -f "$REF/graph_functions.cu" ]; then
    mkdir -p "$SRC" "$SRC48"
    for f in $FILES; do
        cmp -s "$REF/$f" "$SRC/$f" || cp "$REF/$f" "$SRC/$f"
    done
    sed 's/^#define trY 0x00050000/#define trY 0x00300000/' "$SRC/graph_functions.cu" > "$SRC48/graph_functions.cu.new"
    grep -q '^#define trY 0x00300000' "$SRC48/graph_functions.cu.new"
    if cmp -s "$SRC48/graph_functions.cu.new" "$SRC48/graph_functions.cu"; then
        rm -f "$SRC48/graph_functions.cu.new"
    else
        mv "$SRC48/graph_functions.cu.new" "$SRC48/graph_functions.cu"
    fi
elif [ ! -f "$SRC/graph_functions.cu" ]; then
    echo "build_ref: no reference checkout at $REF and no staged copy in $SRC; skipped" >&2
    exit 0
fi

# (re)build a target when it is missing or older than any input
stale() {
    local t="$1"; shift
    [ -f "$t" ] || return 0
    for d in "$@"; do [ "$d" -nt "$t" ] && return 0; done
    return 1
}

pids=()
HOSTFLAGS="-O2 -std=c++14 -fPIC -shared -w -ffp-contract=off"
for y in 5 48; do
    inc="-I$SRC"; [ "$y" = 48 ] && inc="-I$SRC48 -I$SRC"
    t="$OUT/libdepix_ref$y.so"
    if stale "$t" "$HERE/ref_driver.cpp" "$SRC"/*.cu "$SRC48/graph_functions.cu" "$0"; then
        g++ $HOSTFLAGS $inc "$HERE/ref_driver.cpp" -o "$t.tmp" && mv "$t.tmp" "$t" &
        pids+=($!)
    fi
done

NVCC="${CUDA_HOME:-/usr/local/cuda}/bin/nvcc"
[ -x "$NVCC" ] || NVCC="$(command -v nvcc || true)"
if [ "${DEPIX_REF_NO_GPU:-0}" != 1 ] && [ -n "$NVCC" ]; then
    # the reference's NVCCFLAGS (depixel_gpu.pro:48) on sm_103a; FMA
    # contraction is nvcc's default, as in the reference build
    GPUFLAGS="-O3 -use_fast_math -Xcompiler -fno-strict-aliasing -Xcompiler -fPIC -shared -w
              -gencode arch=compute_103a,code=sm_103a"
    for y in 5 48; do
        inc="-I$SRC"; [ "$y" = 48 ] && inc="-I$SRC48 -I$SRC"
        t="$OUT/libdepix_refgpu$y.so"
        if stale "$t" "$HERE/ref_gpu.cu" "$SRC"/*.cu "$SRC48/graph_functions.cu" "$0"; then
            "$NVCC" $GPUFLAGS $inc "$HERE/ref_gpu.cu" -o "$t.tmp" -lcudart && mv "$t.tmp" "$t" &
            pids+=($!)
        fi
    done
fi
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
[ $rc = 0 ] || { echo "build_ref: a build failed" >&2; exit 1; }
echo "build_ref: $(cd "$OUT" && ls lib*.so | tr '\n' ' ')"
