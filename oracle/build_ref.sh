#!/bin/bash
# Builds the reference's own code into oracle/_ref/ for the tests' checks.
# TEST INFRASTRUCTURE ONLY: nothing the product ships links or runs it.
#
# Sources: with LTPMG_REFERENCE pointing at the reference tree, the files the
# checks need (src/, include/, cuda/src/, cuda/include/, data/) are staged
# into oracle/_ref/src/ first -- a build-input copy that git ignores and that
# travels with the working tree to the GPU machine, where the reference tree
# does not exist.  Without LTPMG_REFERENCE the staged copy is used if there is
# one; with neither the script exits 0 without building.
#
# Outputs (all under oracle/_ref/):
#   libltpmg_ref_random.so  the reference's generator pieces (src/random.cpp)
#                           with oracle/ref_harness.cpp, for the golden vectors
#   ltpmg_ref_cuda          the reference's CUDA library (cuda/src/*.cu,
#                           compiled unchanged for sm_103a) with
#                           oracle/ref_cuda_harness.cu: runs the reference's
#                           GPU path on a given batch (needs a GPU to run)
#   ltpmg_ref_gen           the reference's host generator (src/param.cpp,
#                           common.cpp, random.cpp, txn_generator.cpp,
#                           query.cpp) with oracle/ref_gen_harness.cpp: times
#                           Txn_Generator + Query::generate_txn
#   ltpmg_host              the reference's whole host program linked against
#                           this library in place of its CUDA library (when
#                           the library is built)
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
if [ -n "$LTPMG_REFERENCE" ] && [ -f "$LTPMG_REFERENCE/src/random.cpp" ]; then
  rm -rf "$SRC.tmp"
  mkdir -p "$SRC.tmp/cuda"
  cp -r "$LTPMG_REFERENCE/src" "$LTPMG_REFERENCE/include" "$LTPMG_REFERENCE/data" "$SRC.tmp/"
  cp -r "$LTPMG_REFERENCE/cuda/src" "$LTPMG_REFERENCE/cuda/include" "$SRC.tmp/cuda/"
  rm -rf "$SRC"
  mv "$SRC.tmp" "$SRC"
  echo "build_ref: staged the reference sources into $SRC"
fi
if [ ! -f "$SRC/src/random.cpp" ]; then
  echo "build_ref: no reference sources (set LTPMG_REFERENCE to the reference tree); skipping"
  exit 0
fi
mkdir -p "$OUT/obj"
NVCC="${NVCC:-nvcc}"
command -v "$NVCC" >/dev/null 2>&1 || NVCC=/usr/local/cuda/bin/nvcc

g++ -std=c++17 -O2 -fPIC -shared -w \
  -I "$HERE/ref_shim" -I "$SRC/include" \
  "$HERE/ref_harness.cpp" "$SRC/src/random.cpp" \
  -o "$OUT/libltpmg_ref_random.so"
echo "build_ref: built $OUT/libltpmg_ref_random.so"

# the reference's CUDA library, its files compiled in parallel as they are
pids=()
for f in "$SRC"/cuda/src/*.cu "$HERE/ref_cuda_harness.cu"; do
  b="$(basename "$f")"
  "$NVCC" -std=c++20 -O3 -gencode arch=compute_103a,code=sm_103a -w -I "$SRC/cuda/include" \
    -c "$f" -o "$OUT/obj/$b.o" &
  pids+=($!)
done
# the reference's host generator, beside it
g++ -std=c++20 -O2 -w -I "$HERE/ref_shim" -I "$SRC/include" -c "$HERE/ref_gen_harness.cpp" -o "$OUT/obj/gen_harness.o" &
pids+=($!)
for b in param.cpp common.cpp random.cpp txn_generator.cpp query.cpp; do
  g++ -std=c++20 -O2 -w -I "$HERE/ref_shim" -I "$SRC/include" -c "$SRC/src/$b" -o "$OUT/obj/host_$b.o" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" -gencode arch=compute_103a,code=sm_103a "$OUT"/obj/*.cu.o -o "$OUT/ltpmg_ref_cuda" -lpthread
echo "build_ref: built $OUT/ltpmg_ref_cuda"
g++ "$OUT/obj/gen_harness.o" "$OUT"/obj/host_*.o -o "$OUT/ltpmg_ref_gen" -lpthread
echo "build_ref: built $OUT/ltpmg_ref_gen"

# The drop-in check: the reference's whole host program (src/*.cpp, main
# included), with the gflags/glog stand-ins, linked against this library in
# place of its own CUDA library.  Needs the library built first.
LIB_DIR="$(cd "$HERE/.." && pwd)/ltpmg_gb300"
if [ -f "$LIB_DIR/libltpmg_gb300.so" ]; then
  g++ -std=c++20 -O0 -w -I "$HERE/ref_shim" -I "$SRC/include" "$SRC"/src/*.cpp \
    -L "$LIB_DIR" -lltpmg_gb300 -Wl,-rpath,"$LIB_DIR" -lpthread -o "$OUT/ltpmg_host"
  echo "build_ref: linked the reference host program: $OUT/ltpmg_host"
fi
