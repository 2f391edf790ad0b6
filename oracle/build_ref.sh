#!/bin/sh
# Compiles the reference's own C++ sources (where they lie, read-only) into the checker
# binary oracle/_ref/pma_ref, with oracle/ref_shim standing in for FreeImage's file I/O and
# FreeImage's own resize engine (Resize.cpp, Rescale.cpp) compiled over a minimal bitmap. Test
# infrastructure only; needs the reference tree: the first argument, else $PMA_REFERENCE_DIR,
# else /root/reference.
set -e
REF=${1:-${PMA_REFERENCE_DIR:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT/obj"
CXXFLAGS="-std=gnu++98 -fpermissive -w -O2 -fopenmp -DBOOST_DISABLE_ASSERTS -DNDEBUG -I$HERE/ref_shim -I$REF/Externals/Boost -I$REF"
SRCS=$(ls "$REF"/Core/Source/*.cpp "$REF"/ImageProcessing/Main.cpp "$REF"/ImageProcessing/Execution/Source/*.cpp "$REF"/ImageProcessing/Model/Source/*.cpp "$REF"/ImageProcessing/Services/Source/*.cpp)
pids=""
for s in $SRCS; do
  o="$OUT/obj/$(echo "$s" | sed "s|$REF/||; s|/|_|g").o"
  g++ $CXXFLAGS -include sys/types.h -c "$s" -o "$o" &
  pids="$pids $!"
done
# FreeImage's resize engine, from the reference's vendored sources, for the in-plane resampling
FI="$REF/Externals/FreeImage/Source"
FIFLAGS="-O2 -w -ffp-contract=off -I$FI -I$FI/FreeImageToolkit"
for s in "$FI/FreeImageToolkit/Resize.cpp" "$FI/FreeImageToolkit/Rescale.cpp" "$HERE/ref_shim/fi_resize_shim.cpp"; do
  g++ $FIFLAGS -c "$s" -o "$OUT/obj/fi_$(basename "$s" .cpp).o" &
  pids="$pids $!"
done
for p in $pids; do wait $p || exit 1; done
g++ -fopenmp "$OUT"/obj/*.o -o "$OUT/pma_ref"
echo "$OUT/pma_ref"
