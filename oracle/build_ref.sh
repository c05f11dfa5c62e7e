#!/bin/sh
# Builds the checkers under oracle/ (TEST INFRASTRUCTURE ONLY):
#   oracle/_build/libpsi_oracle.so  -- the C restatements (psi_oracle.c: dense
#                                      valuations; psi_sparse.c: path valuations,
#                                      threaded) and the workload generator
#                                      (psi_gen.c), always;
#   oracle/_ref/libpsi_ref.so       -- the reference's own CPUParity, compiled from
#                                      its sources where they lie, when the
#                                      reference tree is present (REF_DIR).
# The reference is compiled from game.cpp and cpu_parity.cpp only (its CMake
# build needs boost and a CUDA 3.5 target, neither used here).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF_DIR=${REF_DIR:-/root/reference}
CC=${CC:-gcc}
CXX=${CXX:-g++}
mkdir -p "$HERE/_build"
$CC -O2 -std=gnu11 -fPIC -shared -pthread -o "$HERE/_build/libpsi_oracle.so" \
    "$HERE/psi_oracle.c" "$HERE/psi_sparse.c" "$HERE/psi_gen.c"
if [ -f "$REF_DIR/cpu_parity.cpp" ] && [ -f "$REF_DIR/game.cpp" ]; then
    mkdir -p "$HERE/_ref"
    $CXX -O2 -std=c++11 -fPIC -shared -pthread -w -I"$REF_DIR" -o "$HERE/_ref/libpsi_ref.so" \
        "$REF_DIR/game.cpp" "$REF_DIR/cpu_parity.cpp" "$HERE/ref_driver.cpp"
    # the reference's own 10-vertex fixture, for the test that pins the ring10 family
    if [ -f "$REF_DIR/test2.gm" ]; then cp "$REF_DIR/test2.gm" "$HERE/_ref/test2.gm"; fi
    # where the sources lie, for the test that compiles the reference-side adapter
    echo "$REF_DIR" > "$HERE/_ref/REF_DIR"
fi
