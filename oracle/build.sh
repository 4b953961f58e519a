#!/bin/bash
# oracle/build.sh -- builds the test-side checkers.  TEST INFRASTRUCTURE ONLY.
#
#   oracle/_ref/liboracle.so     the C restatement (ngia_oracle.c)
#   oracle/_ref/src/             reference sources, staged from the reference
#                                checkout when it is present (NGIA_REFERENCE_DIR,
#                                default: a directory named "reference" beside
#                                the repository's own directory); on machines
#                                without the checkout the staged copy is used
#   oracle/_ref/cpu{,_fma}/      the staged headers with the cuda_stub.h shim
#   oracle/_ref/ngia2_cpu{,_fma} the reference CLI built as a host program
#   oracle/_ref/libngia_ref{,_fma}.so  ref_harness.cpp over the shimmed headers
#   oracle/_ref/ngia2_gpu        the reference CLI, unmodified, built by nvcc
#   oracle/_ref/ref_gpu_align    ref_gpu_harness.cu over the unmodified headers
#
# The *_fma variants replace the two band-bound expressions of the alignment
# kernel by an explicit fused multiply-add, i.e. the rounding of a GPU build
# that contracts them; the plain variants round the product separately.
# Everything under oracle/_ref/ is git-ignored and never part of the product.
#
# usage: oracle/build.sh [--no-gpu]   (--no-gpu skips the two nvcc targets)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
REF="${NGIA_REFERENCE_DIR:-$HERE/../../reference}"
NO_GPU=0
[ "${1:-}" = "--no-gpu" ] && NO_GPU=1
mkdir -p "$OUT"

CFLAGS="-O2 -std=c11 -fPIC -ffp-contract=off"
gcc $CFLAGS -shared "$HERE/ngia_oracle.c" -o "$OUT/liboracle.so.tmp" -lm
mv "$OUT/liboracle.so.tmp" "$OUT/liboracle.so"

# ---- stage the reference sources --------------------------------------------
if [ -f "$REF/src/buildGraph.hpp" ]; then
  mkdir -p "$OUT/src"
  for f in buildGraph.hpp fastClustering.hpp leidenParallel.hpp makedb.hpp \
           parser.hpp saveResult.hpp timer.hpp main.cu; do
    cp -f "$REF/src/$f" "$OUT/src/$f"
    chmod u+w "$OUT/src/$f"
  done
fi
if [ ! -f "$OUT/src/buildGraph.hpp" ]; then
  echo "oracle/build.sh: reference sources not available; built liboracle.so only"
  exit 0
fi

# ---- host (OpenMP) shim of the reference ------------------------------------
shim() {  # $1 = output dir, $2 = 1 for the fused band-bound variant
  local d="$1"
  mkdir -p "$d"
  cp -f "$OUT/src/"*.hpp "$OUT/src/main.cu" "$d/"
  cp -f "$HERE/cuda_stub.h" "$d/"
  for f in buildGraph.hpp fastClustering.hpp; do
    local expr='s|#include <cuda.h>|#include "cuda_stub.h"|; s|kernel_dynamic<<<(count + 63) / 64, 64>>>(|SHIM_LAUNCH(count, kernel_dynamic, |'
    if [ "$2" = 1 ]; then
      expr="$expr;"'s|ceil(lengthTar-lengthTar\*threshold)|ceil(fmaf(-(float)lengthTar, threshold, (float)lengthTar))|; s|ceil(lengthRep-lengthTar\*threshold)|ceil(fmaf(-(float)lengthTar, threshold, (float)lengthRep))|'
    fi
    sed -e "$expr" "$OUT/src/$f" > "$d/$f"
    grep -q 'cuda_stub.h' "$d/$f" || { echo "shim: include not patched in $f"; exit 1; }
    grep -q 'SHIM_LAUNCH(count, kernel_dynamic' "$d/$f" || { echo "shim: launch not patched in $f"; exit 1; }
    if [ "$2" = 1 ]; then
      [ "$(grep -c 'fmaf(' "$d/$f")" = 2 ] || { echo "shim: band bounds not patched in $f"; exit 1; }
    fi
  done
}
shim "$OUT/cpu" 0
shim "$OUT/cpu_fma" 1

HOSTFLAGS="-O3 -std=c++17 -fopenmp -ffp-contract=off -w"
pids=()
g++ $HOSTFLAGS -I"$OUT/cpu" -x c++ "$OUT/cpu/main.cu" -o "$OUT/ngia2_cpu" & pids+=($!)
g++ $HOSTFLAGS -I"$OUT/cpu_fma" -x c++ "$OUT/cpu_fma/main.cu" -o "$OUT/ngia2_cpu_fma" & pids+=($!)
g++ $HOSTFLAGS -fPIC -shared -I"$OUT/cpu" "$HERE/ref_harness.cpp" -o "$OUT/libngia_ref.so" & pids+=($!)
g++ $HOSTFLAGS -fPIC -shared -I"$OUT/cpu_fma" "$HERE/ref_harness.cpp" -o "$OUT/libngia_ref_fma.so" & pids+=($!)

# ---- the reference's own GPU build -------------------------------------------
# The reference Makefile builds with -arch=native; on a GB300 that is sm_103.
if [ "$NO_GPU" = 0 ] && command -v nvcc >/dev/null 2>&1; then
  NVFLAGS="-O3 -Xcompiler -fopenmp -gencode arch=compute_103,code=sm_103 -w"
  nvcc $NVFLAGS "$OUT/src/main.cu" -o "$OUT/ngia2_gpu" & pids+=($!)
  nvcc $NVFLAGS -I"$OUT/src" "$HERE/ref_gpu_harness.cu" -o "$OUT/ref_gpu_align" & pids+=($!)
fi
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
