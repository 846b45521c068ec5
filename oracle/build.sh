#!/usr/bin/env bash
# Builds the oracle (test infrastructure) into oracle/_build/liborc.so.
# -ffp-contract=off keeps every a*b+c un-fused, as rustc does; fma() calls in the
# source are the reference's mul_add sites. No -march flag: the same source and
# flags build on the x86-64 container and the aarch64 GPU host.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
gcc -std=c11 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread \
    -o "$here/_build/liborc.so.tmp" "$here/cpd_oracle.c" -lm
mv "$here/_build/liborc.so.tmp" "$here/_build/liborc.so"
