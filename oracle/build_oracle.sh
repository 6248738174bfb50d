#!/usr/bin/env bash
# Builds oracle/_build/libpg_oracle.so from oracle/pg_oracle.c and oracle/pg_oracle_roar.c (the
# CPU restatements used only by tests, smoke() and bench.py's CPU legs).  Portable: no
# -march=native, no intrinsics.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
arch_flags=""
case "$(uname -m)" in
  x86_64) arch_flags="-mfma" ;;  # hardware fmaf; results are identical to the libm fmaf
esac
gcc -O3 -std=c11 -fPIC -shared -fopenmp -ffp-contract=off $arch_flags \
  -o "$here/_build/libpg_oracle.so.tmp" "$here/pg_oracle.c" "$here/pg_oracle_roar.c" -lm
mv "$here/_build/libpg_oracle.so.tmp" "$here/_build/libpg_oracle.so"
echo "$here/_build/libpg_oracle.so"
