#!/usr/bin/env bash
# Copy the reference's CUDA backend sources (kernels, host driver, vendored IO headers,
# training_config.json) and its PyTorch extension's CUDA bindings from the read-only
# reference checkout into baseline/_ref/, the git-ignored location of the reference that is
# copied with the working tree to the machine with the GPU.  Nothing here is committed;
# oracle/ref/build.sh compiles from that copy.
#   usage: oracle/ref/stage.sh [/path/to/reference]
set -euo pipefail
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")/../.." && pwd)
DST="$HERE/baseline/_ref/sad"
rm -rf "$DST"
mkdir -p "$DST"
cp -r "$REF/backends/cuda/src" "$DST/src"
cp -r "$REF/backends/cuda/third_party" "$DST/third_party"
cp "$REF/training_config.json" "$DST/"
# the PyTorch extension's CUDA bindings (render_sad / render_sad_backward and the rest)
mkdir -p "$DST/torch_ext"
cp "$REF/backends/pytorch/torch_ext/torch_binding.cpp" "$REF/backends/pytorch/torch_ext/torch_binding.h" "$DST/torch_ext/"
cp -r "$REF/backends/pytorch/torch_ext/cuda" "$DST/torch_ext/cuda"
echo "staged $(ls "$DST/src" | wc -l) files into $DST"
