#!/usr/bin/env bash
# Entry point with the reference's run.sh interface:
#   ./run.sh <image.png | image directory> [--backend auto|cuda] [sad_cuda options]
#   ./run.sh --render <sites.txt> [--backend auto|cuda] [render options]
# Only the CUDA backend exists here (sad_gb300/_lib/sad_cuda on libsad_gb300); it is built
# on first use and rebuilt when a source under sad_gb300/ or include/ is newer.  The
# defaults come from $CONFIG_PATH (default: the packaged sad_gb300/training_config.json).
set -euo pipefail

ROOT_DIR="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
cd "$ROOT_DIR"
CUDA_BIN="$ROOT_DIR/sad_gb300/_lib/sad_cuda"
export CONFIG_PATH="${CONFIG_PATH:-$ROOT_DIR/sad_gb300/training_config.json}"

backend="auto"
args=()
while [ $# -gt 0 ]; do
    case "$1" in
        --backend=*) backend="${1#*=}"; shift ;;
        --backend)
            if [ $# -lt 2 ]; then echo "Missing value for --backend"; exit 1; fi
            backend="$2"; shift 2 ;;
        *) args+=("$1"); shift ;;
    esac
done

case "$backend" in
    auto|cuda) ;;
    *) echo "Backend '$backend' is not part of this build (available: cuda)."; exit 1 ;;
esac

if [ ! -x "$CUDA_BIN" ] || find "$ROOT_DIR/sad_gb300" "$ROOT_DIR/include" -type f \
        \( -name '*.cu' -o -name '*.cuh' -o -name '*.cpp' -o -name '*.h' \) -newer "$CUDA_BIN" | grep -q .; then
    python3 -c "from sad_gb300 import build; build.build()" > /dev/null
fi

# --render, --help and option-only calls go straight to the binary
if [ ${#args[@]} -eq 0 ] || [[ "${args[0]}" == --* ]] || [ "${args[0]}" = "-h" ]; then
    if [ ${#args[@]} -eq 0 ] && [ -f "$ROOT_DIR/test.png" ]; then
        args=("$ROOT_DIR/test.png")
    fi
    exec "$CUDA_BIN" ${args[@]+"${args[@]}"}
fi

input="${args[0]}"
extra=("${args[@]:1}")
if [ ! -d "$input" ]; then
    exec "$CUDA_BIN" "$input" ${extra[@]+"${extra[@]}"}
fi

# Batch mode: every png/jpg/jpeg directly inside the directory, one fit each, with a
# summary log (<out-dir>/batch_<timestamp>.log) of duration, last PSNR and active sites.
images=()
while IFS= read -r -d '' f; do
    images+=("$f")
done < <(find "$input" -maxdepth 1 -type f \( -iname '*.png' -o -iname '*.jpg' -o -iname '*.jpeg' \) -print0 | sort -z)
if [ ${#images[@]} -eq 0 ]; then
    echo "No image files found in directory: $input"
    echo "Supported formats: png, jpg, jpeg"
    exit 1
fi
out_dir="results"
for ((i = 0; i < ${#extra[@]}; i++)); do
    case "${extra[$i]}" in
        --out-dir) if [ $((i + 1)) -lt ${#extra[@]} ]; then out_dir="${extra[$((i + 1))]}"; fi; break ;;
        --out-dir=*) out_dir="${extra[$i]#*=}"; break ;;
    esac
done
mkdir -p "$out_dir"
batch_log="$(cd "$out_dir" && pwd)/batch_$(date +%Y%m%d_%H%M%S).log"
{
    echo "Batch processing log - $(date)"
    echo "Input directory: $input"
    echo "Output directory: $out_dir"
    echo "Backend: cuda"
    echo "Total images: ${#images[@]}"
    echo "==========================================="
} > "$batch_log"
echo "Found ${#images[@]} image(s) in $input"
echo "Batch log: $batch_log"

for img in "${images[@]}"; do
    echo "Processing: $img"
    t0=$(date +%s)
    out_txt="$(mktemp)"
    set +e
    "$CUDA_BIN" "$img" ${extra[@]+"${extra[@]}"} 2>&1 | tee "$out_txt"
    rc=${PIPESTATUS[0]}
    set -e
    {
        echo ""
        echo "Image: $(basename "$img")"
        echo "Duration: $(( $(date +%s) - t0 ))s"
        psnr="$(grep -i psnr "$out_txt" | tail -1 | grep -oE '[0-9]+\.[0-9]+' | head -1 || true)"
        sites="$(grep -i active "$out_txt" | tail -1 | grep -oE '[0-9]+/[0-9]+' | head -1 || true)"
        if [ -n "$psnr" ]; then echo "PSNR: $psnr dB"; fi
        if [ -n "$sites" ]; then echo "Active sites: $sites"; fi
        if [ "$rc" -eq 0 ]; then echo "Status: SUCCESS"; else echo "Status: FAILED (exit code: $rc)"; fi
        echo "-------------------------------------------"
    } >> "$batch_log"
    rm -f "$out_txt"
    if [ "$rc" -ne 0 ]; then
        echo "Error processing $img"
        {
            echo ""
            echo "BATCH PROCESSING FAILED at image: $(basename "$img")"
            echo "Batch log saved to: $batch_log"
        } >> "$batch_log"
        exit 1
    fi
    echo ""
done
echo "Batch processing complete."
echo "Processed ${#images[@]} image(s) successfully."
echo "Batch log: $batch_log"
