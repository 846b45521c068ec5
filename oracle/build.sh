#!/usr/bin/env bash
# Builds the oracle (test infrastructure) into oracle/_build/liborc.so.
# -ffp-contract=off keeps every a*b+c un-fused, as rustc does; fma() calls in the
# source are the reference's mul_add sites. -O3, and on the Arm GPU host the Grace core
# type (the reference builds with target-cpu=native, pyproject.toml:21): vector code of
# the same IEEE operations, so the results do not change; the x86-64 container builds the
# same source with -O3 alone.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
flags=(-std=c11 -O3 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread)
if [ "$(uname -m)" = "aarch64" ] && echo 'int main(void){return 0;}' | gcc -mcpu=neoverse-v2 -x c - -o /dev/null 2>/dev/null; then
    flags+=(-mcpu=neoverse-v2)
fi
gcc "${flags[@]}" -o "$here/_build/liborc.so.tmp" "$here/cpd_oracle.c" "$here/cpd_oracle_toric.c" -lm
mv "$here/_build/liborc.so.tmp" "$here/_build/liborc.so"
# the op-counting build of the same model (the frozen per-ray operation table)
g++ -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -Wno-class-memaccess \
    -o "$here/_build/liborc_ops.so.tmp" "$here/ops_count.cpp"
mv "$here/_build/liborc_ops.so.tmp" "$here/_build/liborc_ops.so"
