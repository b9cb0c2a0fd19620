#!/usr/bin/env bash
# Compile, from the staged copy in baseline/_ref/sad, (1) the reference's kernel files
# linked with oracle/ref/harness.cu into oracle/_ref/ref_harness and (2) the reference's
# CLI (sad_cuda.cu + kernels) into oracle/_ref/sad_cuda.  nvcc only, no cmake; outputs go
# to oracle/_ref/ only.  The CLI is built with STBIR_NO_SIMD: nvcc's host front end cannot
# parse the NEON intrinsics stb_image_resize selects on aarch64.  A CLI build failure does
# not stop the harness build (exit status 3 reports it).
set -uo pipefail
HERE=$(cd "$(dirname "$0")/../.." && pwd)
SRC="$HERE/baseline/_ref/sad/src"
TP="$HERE/baseline/_ref/sad/third_party"
# REF_OUT / REF_ARCH select another output folder under oracle/_ref and another target,
# e.g. REF_ARCH="-gencode arch=compute_86,code=compute_86" for the reference's shipped
# sm_86 PTX, compiled by the CUDA driver when the program loads.
OUT="${REF_OUT:-$HERE/oracle/_ref}"
ARCH="${REF_ARCH:--gencode arch=compute_103a,code=sm_103a}"
mkdir -p "$OUT"
KERNELS="render jfa candidate_pack gradients adam tau_diffusion densify_prune radix_sort utils"
pids=()
for k in $KERNELS; do
  nvcc $ARCH -O3 -std=c++17 -I"$SRC" -c "$SRC/$k.cu" -o "$OUT/$k.o" & pids+=($!)
done
nvcc $ARCH -O3 -std=c++17 -I"$SRC" -c "$HERE/oracle/ref/harness.cu" -o "$OUT/harness.o" & pids+=($!)
nvcc $ARCH -O3 -std=c++17 --extended-lambda -DSTBIR_NO_SIMD -I"$SRC" -I"$TP" \
  -c "$SRC/sad_cuda.cu" -o "$OUT/sad_cuda_main.o" > "$OUT/sad_cuda_build.log" 2>&1 &
cli_pid=$!
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
[ $rc -eq 0 ] || { echo "reference kernel build failed" >&2; exit 1; }
objs=""
for k in $KERNELS; do objs="$objs $OUT/$k.o"; done
nvcc $ARCH -o "$OUT/ref_harness" "$OUT/harness.o" $objs || exit 1
echo "built $OUT/ref_harness"
if wait "$cli_pid" && nvcc $ARCH -o "$OUT/sad_cuda" "$OUT/sad_cuda_main.o" $objs; then
  echo "built $OUT/sad_cuda"
else
  echo "reference CLI build failed (see $OUT/sad_cuda_build.log)" >&2
  tail -20 "$OUT/sad_cuda_build.log" >&2
  exit 3
fi
