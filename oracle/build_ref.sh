#!/bin/sh
# Builds oracle/_ref/libmacis_ref.so from the reference's own MACIS sources
# where they lie (read-only, never copied), plus the project-written API shims
# in oracle/ref_shims and the C-ABI driver oracle/macis_ref.cpp.  Test
# infrastructure: it runs the reference's unmodified code to produce golden
# fixtures (tests/golden/make_ref_golden.py).  Needs the reference checkout;
# usage: sh oracle/build_ref.sh REFERENCE_CHECKOUT
set -e
REF=${1:-$QDK_REFERENCE}
test -n "$REF" || { echo "usage: sh oracle/build_ref.sh REFERENCE_CHECKOUT" >&2; exit 2; }
MACIS="$REF/external/macis"
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
test -d "$MACIS/include/macis" || { echo "reference MACIS not found under $MACIS" >&2; exit 2; }
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-std=c++20 -O3 -fopenmp -fPIC -w -DNDEBUG"
INC="-I$HERE/ref_shims -I$MACIS/include -I$MACIS/src/sparsexx/include -I$MACIS/src/lobpcgxx/include"
# base.cxx: the reference's explicit instantiation of HamiltonianGeneratorBase
# (integral intermediates, fast diagonals)
$CXX $FLAGS $INC -c "$MACIS/src/macis/hamiltonian_generator/base.cxx" -o "$OUT/base.o" &
# transform.cxx: integral transforms that asci_grow's orbital-rotation branch links
$CXX $FLAGS $INC -c "$MACIS/src/macis/transform.cxx" -o "$OUT/transform.o" &
$CXX $FLAGS $INC -c "$HERE/macis_ref.cpp" -o "$OUT/macis_ref.o" &
wait
$CXX -shared -fopenmp -Wl,--no-undefined -o "$OUT/libmacis_ref.so" "$OUT/base.o" "$OUT/transform.o" \
  "$OUT/macis_ref.o"
echo "$OUT/libmacis_ref.so"
