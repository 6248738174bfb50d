#!/usr/bin/env bash
# Builds oracle/_ref/libref_search.so: the reference's own beam-search kernels
# (link_process_v0_store_base_data and search_shared_hashtable in include/Gsearcher.cuh, compiled
# where they lie in the reference tree) under the 32-lane warp emulator of oracle/ref_warp_emu.h,
# instantiated by oracle/ref_search_harness.cpp.  x86-64 only (the emulator's fiber switch).
# Test infrastructure only; the output stays in oracle/_ref/ (git-ignored).
# Usage: oracle/build_ref_search.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $PG_REFERENCE_ROOT, else the checkout named "reference" beside
#   this repository.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-${PG_REFERENCE_ROOT:-$(dirname "$(dirname "$here")")/reference}}"
if [ ! -f "$ref/include/Gsearcher.cuh" ]; then
  echo "reference tree not found at $ref" >&2
  exit 2
fi
if [ "$(uname -m)" != "x86_64" ]; then
  echo "the warp emulator's fiber switch is x86-64 code" >&2
  exit 3
fi
mkdir -p "$here/_ref"
# -DNDEBUG: the reference's release flags (CMakeLists.txt:40) compile its device asserts out.
# -ffp-contract=fast -mfma: sum += x*y becomes one fused multiply-add, as nvcc compiles it.
# -fwrapv: (1 << lane_id) - 1 at lane 31 wraps as the GPU's integer arithmetic does
#   (Gsearcher.cuh:97).
g++ -O2 -std=c++17 -fPIC -shared -DNDEBUG -ffp-contract=fast -mfma -fwrapv \
  -I"$ref/include" -I/usr/local/cuda/include \
  -o "$here/_ref/libref_search.so" "$here/ref_search_harness.cpp" -w
echo "$here/_ref/libref_search.so"
