#!/usr/bin/env bash
# Builds oracle/_ref/libref_harness.so: the reference's own kernel templates (include/Gbuilder.cuh,
# include/Ghashtable.cuh, compiled where they lie under the reference tree) instantiated by
# oracle/ref_harness.cpp for a one-thread CPU run.  Test infrastructure only; the output stays in
# oracle/_ref/ (git-ignored).  Usage: oracle/build_ref.sh [REFERENCE_ROOT] [N] [D]
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-${PG_REFERENCE_ROOT:-$(dirname "$(dirname "$here")")/reference}}"
n="${2:-1000}"
d="${3:-200}"
if [ ! -f "$ref/include/Gbuilder.cuh" ]; then
  echo "reference tree not found at $ref" >&2
  exit 2
fi
mkdir -p "$here/_ref"
arch_flags=""
case "$(uname -m)" in
  x86_64) arch_flags="-mfma" ;;  # hardware FMA so that g++ contracts sum += x*y like nvcc does
esac
# -DNDEBUG: the reference's release flags (CMakeLists.txt:40) compile its device asserts out.
# -ffp-contract=fast: contract a*b+c into one fused multiply-add, as nvcc does by default.
g++ -O2 -std=c++17 -fPIC -shared -DNDEBUG -ffp-contract=fast $arch_flags \
  -DREF_N="$n" -DREF_D="$d" \
  -include "$here/ref_shim.h" -I"$ref/include" -I/usr/local/cuda/include \
  -o "$here/_ref/libref_harness_${n}_${d}.so" "$here/ref_harness.cpp" -w
echo "$here/_ref/libref_harness_${n}_${d}.so"
