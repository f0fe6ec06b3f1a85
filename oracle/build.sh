#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/liboracle.so.
# binary32 arithmetic must not be contracted into FMAs: -ffp-contract=off.
# No -march flags: the same recipe runs on x86_64 and aarch64 hosts.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="${HERE}/liboracle.so"
${CC:-gcc} -std=c11 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread \
  -Wall -Wno-unused-function -o "${OUT}.tmp" "${HERE}/rt_oracle.c" -lm
mv -f "${OUT}.tmp" "${OUT}"
echo "built ${OUT}"
