#!/usr/bin/env bash
# Builds oracle/_ref/libref_cpu.so: the reference's CPU RoarGraph functions (compare, MatchNN,
# MatchSup, FusionNN, FusionFinal in tests/test_t2iend.cu, compiled where it lies) wrapped by
# oracle/ref_cpu_harness.cu.  x86-64 with AVX-512 only (the reference's compare is AVX-512 code).
# Test infrastructure only; the output stays in oracle/_ref/ (git-ignored).
# Usage: oracle/build_ref_cpu.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $PG_REFERENCE_ROOT, else the checkout named "reference" beside
#   this repository.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-${PG_REFERENCE_ROOT:-$(dirname "$(dirname "$here")")/reference}}"
if [ ! -f "$ref/tests/test_t2iend.cu" ]; then
  echo "reference tree not found at $ref" >&2
  exit 2
fi
if [ "$(uname -m)" != "x86_64" ] || ! grep -q avx512f /proc/cpuinfo; then
  echo "the reference's CPU path needs an x86-64 host with AVX-512" >&2
  exit 3
fi
mkdir -p "$here/_ref"
# host flags follow the reference's release build (CMakeLists.txt:36-38: -O3, OpenMP, NDEBUG);
# AVX-512 is enabled explicitly instead of -march=native so the build does not depend on the host
nvcc -x cu -std=c++17 -O3 -shared -Xcompiler -fPIC,-fopenmp,-O3,-DNDEBUG,-mavx512f,-mavx512dq,-mfma,-mavx2 \
  -gencode arch=compute_103a,code=compute_103a \
  -I"$here/ref_stub" -I"$ref/include" -I"$ref/tests" \
  -o "$here/_ref/libref_cpu.so" "$here/ref_cpu_harness.cu" -lgomp -w
echo "$here/_ref/libref_cpu.so"
