#!/bin/bash
# ORACLE recipe (test infrastructure): compile the reference's own, unmodified
# SyncPrims CUDA sources into device-code modules under oracle/_ref/.
#
# The reference tree exists only in the build container, so the modules are
# built here and travel to the GPU machine with the rest of the working tree;
# oracle/ref_runner.cpp (built on the GPU machine) loads and launches them there with
# the reference's own launch shape.  Nothing from /root/reference is copied
# into the repository: only compiler output lands in oracle/_ref/ (git-ignored).
#
#   syncprims_t32_sm100.cubin    stock sources, NUM_THREADS_PER_BLOCK 32 (main.cu:8)
#   syncprims_t256_sm100.cubin   same sources with main.cu:8 set to 256, compiled
#                                from a temporary copy (the semaphore kernels size
#                                a shared array by it, main.cu:567)
# Both with -DHAS_NANOSLEEP=1 (Makefile:10) for sm_100, the architecture the
# reference would be built for on Blackwell (its Makefile's compute_60..80 list is
# rejected by CUDA 13).
set -euo pipefail
REF=${HS_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SP="$REF/cuda/syncPrims/uvm"
# without the reference tree (the GPU machine) the modules built here are used as they are
[ -f "$SP/main.cu" ] || { [ -n "${HS_REQUIRE_REFERENCE:-}" ] && { echo "reference tree not found at $REF" >&2; exit 1; }; exit 0; }
mkdir -p "$OUT"
NVCC=${NVCC:-nvcc}
GEN="-gencode arch=compute_100,code=sm_100"
newest=$(ls -t "$SP"/*.cu "$SP"/*.h | head -1)

build() {  # $1 = output, $2 = main source, $3.. = extra flags
  local out="$1" src="$2"; shift 2
  if [ -f "$out" ] && [ "$out" -nt "$newest" ] && [ "$out" -nt "$0" ]; then return 0; fi
  "$NVCC" -cubin $GEN -O3 -DHAS_NANOSLEEP=1 "$@" "$src" -o "$out"
}

build "$OUT/syncprims_t32_sm100.cubin" "$SP/main.cu"
TMP=$(mktemp -d)
trap 'rm -rf "$TMP"' EXIT
sed 's/^#define NUM_THREADS_PER_BLOCK 32$/#define NUM_THREADS_PER_BLOCK 256/' "$SP/main.cu" > "$TMP/main.cu"
grep -q '^#define NUM_THREADS_PER_BLOCK 256$' "$TMP/main.cu"
build "$OUT/syncprims_t256_sm100.cubin" "$TMP/main.cu" -I"$SP"
echo "reference modules in $OUT"
