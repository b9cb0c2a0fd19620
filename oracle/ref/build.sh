#!/usr/bin/env bash
# Compile, from the staged copy in baseline/_ref/sad, (1) the reference's kernel files
# linked with oracle/ref/harness.cu into oracle/_ref/ref_harness and (2) the reference's
# CLI (sad_cuda.cu + kernels) into oracle/_ref/sad_cuda.  nvcc only, no cmake; outputs go
# to oracle/_ref/ only.
set -euo pipefail
HERE=$(cd "$(dirname "$0")/../.." && pwd)
SRC="$HERE/baseline/_ref/sad/src"
TP="$HERE/baseline/_ref/sad/third_party"
OUT="$HERE/oracle/_ref"
ARCH="-gencode arch=compute_103a,code=sm_103a"
mkdir -p "$OUT"
KERNELS="render jfa candidate_pack gradients adam tau_diffusion densify_prune radix_sort utils"
pids=()
for k in $KERNELS; do
  nvcc $ARCH -O3 -std=c++17 -I"$SRC" -c "$SRC/$k.cu" -o "$OUT/$k.o" & pids+=($!)
done
nvcc $ARCH -O3 -std=c++17 -I"$SRC" -c "$HERE/oracle/ref/harness.cu" -o "$OUT/harness.o" & pids+=($!)
nvcc $ARCH -O3 -std=c++17 --extended-lambda -I"$SRC" -I"$TP" -c "$SRC/sad_cuda.cu" -o "$OUT/sad_cuda_main.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
objs=""
for k in $KERNELS; do objs="$objs $OUT/$k.o"; done
nvcc $ARCH -o "$OUT/ref_harness" "$OUT/harness.o" $objs
nvcc $ARCH -o "$OUT/sad_cuda" "$OUT/sad_cuda_main.o" $objs
echo "built $OUT/ref_harness $OUT/sad_cuda"
