#!/usr/bin/env bash
# Render a saved sites file (TXT or JSON) through run.sh, e.g.
#   ./render.sh results/foo_sites.txt --width 1024 --height 1024
set -euo pipefail
ROOT_DIR="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
exec "$ROOT_DIR/run.sh" --render "$@"
