#!/bin/bash
# Builds the reference's own host generator code (src/random.cpp) together
# with oracle/ref_harness.cpp into oracle/_ref/ for the golden-vector script.
# Test infrastructure only.  Reads the reference sources where they lie and
# writes nothing but oracle/_ref/.  Exits 0 without building when the
# reference tree is absent (it is not present on the GPU machines).
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${LTPMG_REFERENCE:-/root/reference}"
if [ ! -f "$REF/src/random.cpp" ]; then
  echo "build_ref: reference sources not found at $REF; skipping"
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O2 -fPIC -shared -w \
  -I "$HERE/ref_shim" -I "$REF/include" \
  "$HERE/ref_harness.cpp" "$REF/src/random.cpp" \
  -o "$HERE/_ref/libltpmg_ref_random.so"
echo "build_ref: built $HERE/_ref/libltpmg_ref_random.so"
