#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_ref/liboracle.so.
# -ffp-contract=off: no fused multiply-add, matching Julia's evaluation.
# OpenMP parallelises only row loops whose per-row arithmetic is unchanged,
# so results do not depend on the thread count.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_ref"
flags=(-O2 -std=c11 -fPIC -shared -ffp-contract=off -fno-fast-math -Wall -Wno-unused-function -Wno-maybe-uninitialized)
if echo 'int main(void){return 0;}' | gcc -fopenmp -x c - -o /dev/null 2>/dev/null; then
  flags+=(-fopenmp)
fi
gcc "${flags[@]}" "$here/cpdlp_oracle.c" -o "$here/_ref/liboracle.so.tmp" -lm
mv "$here/_ref/liboracle.so.tmp" "$here/_ref/liboracle.so"
