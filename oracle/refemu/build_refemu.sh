#!/bin/sh
# Builds oracle/_ref/librefemu.so: the reference's own kernel sources
# (LB_kernel.cu, which includes sem_kernel.cu) compiled with g++ through the
# serial CUDA emulation header, plus the step-loop harness refemu.cpp.
# Oracle test infrastructure: it reads the reference tree, so it only builds
# where that tree is present (REF_DIR, default: a `reference` directory
# beside the repository checkout).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF_DIR=${REF_DIR:-$HERE/../../../reference}
OUT="$HERE/../_ref"
if [ ! -f "$REF_DIR/LB_kernel.cu" ]; then
  echo "reference tree not found at $REF_DIR; skipping refemu build" >&2
  exit 0
fi
mkdir -p "$OUT"
g++ -O2 -std=c++17 -fPIC -shared -w -fno-fast-math -ffp-contract=off \
    -x c++ -I"$HERE/stub" -I"$HERE" -I"$REF_DIR" \
    "$HERE/refemu.cpp" -o "$OUT/librefemu.so"
echo "built $OUT/librefemu.so"
# the driver's host code with stub GPU entry points (refhost_driver.c)
gcc -O1 -std=gnu11 -fPIC -shared -w -fno-fast-math -ffp-contract=off \
    -I"$HERE/stub" -I"$HERE" -I"$REF_DIR" \
    "$HERE/refhost_driver.c" -o "$OUT/librefhost_driver.so" -lm
echo "built $OUT/librefhost_driver.so"
# the fibrin code's worm-like-chain law (refhost_fiber.cpp)
g++ -O1 -std=c++17 -fPIC -shared -w -fno-fast-math -ffp-contract=off \
    -I"$HERE/stub" -I"$HERE" -I"$REF_DIR" \
    "$HERE/refhost_fiber.cpp" "$REF_DIR/network.cpp" -o "$OUT/librefhost_fiber.so"
echo "built $OUT/librefhost_fiber.so"
