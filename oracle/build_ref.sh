#!/bin/sh
# Test infrastructure only. Compiles the REFERENCE solver from its own sources,
# read where they lie (never copied), plus oracle/ref_harness.cpp, into
# oracle/_ref/ref_solve. The reference's kernels are AVX-512 intrinsics
# (MatrixStdDouble.cpp), so this builds only on an x86-64 host with AVX-512;
# on any other host it exits 0 after saying why, and the C restatement in
# oracle/soglu_oracle.c is the only CPU oracle there.
#
# Flags follow the reference Makefile (Makefile:5): -std=c++11 -O3 -Ofast
# -fopenmp -fpermissive -mprefer-vector-width=512, with -march=native in place
# of the hard-coded -march=skylake-avx512 and g++ in place of g++-9.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${SOGLU_REFERENCE_DIR:-/root/reference}
OUT="$HERE/_ref"
if [ ! -f "$REF/MatrixStdDouble.cpp" ]; then
    echo "build_ref: reference sources not present at $REF; skipped"; exit 0
fi
if ! grep -q avx512f /proc/cpuinfo 2>/dev/null; then
    echo "build_ref: host has no AVX-512; the reference kernels cannot compile here; skipped"; exit 0
fi
mkdir -p "$OUT/obj"
CXX=${CXX:-g++}
FLAGS="-std=c++11 -O3 -Ofast -march=native -fopenmp -fpermissive -mprefer-vector-width=512 -pthread -w"
for f in BlockPlanner GPSOrder MatrixStdDouble config data matrix memutil mtx operation solver; do
    if [ ! -f "$OUT/obj/$f.o" ] || [ "$REF/$f.cpp" -nt "$OUT/obj/$f.o" ]; then
        $CXX -c $FLAGS -I"$REF" "$REF/$f.cpp" -o "$OUT/obj/$f.o" &
    fi
done
wait
$CXX $FLAGS -I"$REF" "$HERE/ref_harness.cpp" "$OUT"/obj/*.o -o "$OUT/ref_solve" -lm
echo "build_ref: built $OUT/ref_solve"
