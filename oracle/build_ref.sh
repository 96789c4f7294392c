#!/bin/bash
# ORACLE recipe (test infrastructure): compile the reference's own, unmodified
# SyncPrims CUDA sources into device-code modules under oracle/_ref/.
#
# The reference tree is found through HS_REFERENCE_DIR, else as a checkout
# named "reference" beside this repository.  Where it is absent (a machine that
# only runs the modules) the modules already in oracle/_ref/ are used as they
# are; oracle/ref_runner.cpp loads and launches them with the reference's own
# launch shape.  Nothing of the reference's source is copied into the
# repository: only compiler output lands in oracle/_ref/ (git-ignored).
#
#   syncprims_t32_sm100.cubin    stock sources, NUM_THREADS_PER_BLOCK 32 (main.cu:8)
#   syncprims_t256_sm100.cubin   same sources with main.cu:8 set to 256, compiled
#                                from a temporary copy (the semaphore kernels size
#                                a shared array by it, main.cu:567)
#   refcounter_sm100.cubin       cuda/relaxedAtomics/uvm/refCounter/refCounter_kernel.cu
#                                (the other relaxed-atomics kernels are not built:
#                                splitCounter's readers reach __syncthreads in
#                                divergent half-warps, seqlocks' readers likewise,
#                                flags overruns randArr -- none is run here)
# Both with -DHAS_NANOSLEEP=1 (Makefile:10) for sm_100, the architecture the
# reference would be built for on Blackwell (its Makefile's compute_60..80 list is
# rejected by CUDA 13).
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${HS_REFERENCE_DIR:-$HERE/../../reference}
OUT="$HERE/_ref"
SP="$REF/cuda/syncPrims/uvm"
# without the reference tree (the GPU machine) the modules built here are used as they are
[ -f "$SP/main.cu" ] || { [ -n "${HS_REQUIRE_REFERENCE:-}" ] && { echo "reference tree not found at $REF" >&2; exit 1; }; exit 0; }
mkdir -p "$OUT"
NVCC=${NVCC:-nvcc}
GEN="-gencode arch=compute_100,code=sm_100"
RC="$REF/cuda/relaxedAtomics/uvm/refCounter"
newest=$(ls -t "$SP"/*.cu "$SP"/*.h "$RC"/*.cu | head -1)

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
build "$OUT/refcounter_sm100.cubin" "$RC/refCounter_kernel.cu"
echo "reference modules in $OUT"
