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

# The drop-in check: the reference's whole host program (src/*.cpp, main
# included), with the gflags/glog stand-ins, linked against this library in
# place of its own CUDA library.  Needs the library built first.
LIB_DIR="$(cd "$HERE/.." && pwd)/ltpmg_gb300"
if [ -f "$LIB_DIR/libltpmg_gb300.so" ]; then
  g++ -std=c++20 -O0 -w -I "$HERE/ref_shim" -I "$REF/include" "$REF"/src/*.cpp \
    -L "$LIB_DIR" -lltpmg_gb300 -Wl,-rpath,"$LIB_DIR" -lpthread -o "$HERE/_ref/ltpmg_host"
  echo "build_ref: linked the reference host program: $HERE/_ref/ltpmg_host"
fi
