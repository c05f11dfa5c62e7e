#!/bin/sh
# Builds the checkers under oracle/ (TEST INFRASTRUCTURE ONLY):
#   oracle/_build/libpsi_oracle.so  -- the C restatements (psi_oracle.c: dense
#                                      valuations; psi_sparse.c: path valuations,
#                                      threaded; psi_bf.c: the Bellman-Ford best
#                                      response) and the workload generator
#                                      (psi_gen.c), always;
#   oracle/_ref/libpsi_ref.so       -- the reference's own CPUParity, compiled from
#                                      its sources where they lie, when the
#                                      reference tree is present (REF_DIR);
#   oracle/_ref/libpsi_refbf.so     -- the reference's own CPU_BellmanFord, likewise.
# CPUParity is compiled from game.cpp and cpu_parity.cpp, CPU_BellmanFord from
# game.cpp, valuation.cpp, cpu_bv.cpp and cpu_bf.cpp, and nothing else: the
# reference's CMake build needs boost and a CUDA 3.5 target, neither used here.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF_DIR=${REF_DIR:-/root/reference}
CC=${CC:-gcc}
CXX=${CXX:-g++}
mkdir -p "$HERE/_build"
$CC -O2 -std=gnu11 -fPIC -shared -pthread -o "$HERE/_build/libpsi_oracle.so" \
    "$HERE/psi_oracle.c" "$HERE/psi_sparse.c" "$HERE/psi_gen.c" "$HERE/psi_bf.c"
if [ -f "$REF_DIR/cpu_parity.cpp" ] && [ -f "$REF_DIR/game.cpp" ]; then
    mkdir -p "$HERE/_ref"
    $CXX -O2 -std=c++11 -fPIC -shared -pthread -w -I"$REF_DIR" -o "$HERE/_ref/libpsi_ref.so" \
        "$REF_DIR/game.cpp" "$REF_DIR/cpu_parity.cpp" "$HERE/ref_driver.cpp"
    if [ -f "$REF_DIR/cpu_bf.cpp" ] && [ -f "$REF_DIR/cpu_bv.cpp" ] && [ -f "$REF_DIR/valuation.cpp" ]; then
        $CXX -O2 -std=c++11 -fPIC -shared -pthread -w -I"$REF_DIR" -o "$HERE/_ref/libpsi_refbf.so" \
            "$REF_DIR/game.cpp" "$REF_DIR/valuation.cpp" "$REF_DIR/cpu_bv.cpp" "$REF_DIR/cpu_bf.cpp" \
            "$HERE/ref_bf_driver.cpp"
    fi
    # the reference's own 10-vertex fixture, for the test that pins the ring10 family
    if [ -f "$REF_DIR/test2.gm" ]; then cp "$REF_DIR/test2.gm" "$HERE/_ref/test2.gm"; fi
    # where the sources lie, for the test that compiles the reference-side adapter
    echo "$REF_DIR" > "$HERE/_ref/REF_DIR"
fi
