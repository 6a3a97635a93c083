#!/usr/bin/env bash
# Builds the C oracle (test infrastructure) into oracle/_build/libasdpocs_oracle.so.
# -ffp-contract=off: every float operation rounds as written, matching the
# reference's expression order without fused multiply-adds.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$HERE/_build"
"${CC:-gcc}" -O2 -fPIC -shared -fopenmp -ffp-contract=off -std=c11 \
  -o "$HERE/_build/libasdpocs_oracle.so" "$HERE/asdpocs_oracle.c" -lm
echo "build_oracle: built $HERE/_build/libasdpocs_oracle.so"
