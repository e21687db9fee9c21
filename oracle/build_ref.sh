#!/bin/sh
# Builds the reference-derived checkers into oracle/_ref/ (git-ignored), from
# the reference's sources where they lie: REF_DIR, or else baseline/_ref (the
# unmodified files oracle/stage_ref.sh placed there); nothing is copied.  Test
# infrastructure and the reference arm of bench.py only.
#
#   _ref/libdymref.so   the reference's group.c, lattice.c and dym-mod-metro.cpp
#                       (main renamed) + oracle/ref_harness.cpp, no OpenMP so
#                       every sum runs in the reference's serial order
#   _ref/dym-mod-metro  the unmodified reference executable, built with the
#                       flags of the reference Makefile (-O3 -g -pg -fopenmp)
#   _ref/dym-mod-metro-nhit10   the same with NHIT 10 instead of 20: the source
#                       is streamed through sed into the compiler (no copy)
#   _ref/llr            the unmodified LLR window-ladder executable (llr.cpp),
#                       reference Makefile flags
#   _ref/llr2d          the unmodified two-dimensional LLR executable
#                       (llr2d.cpp), reference Makefile flags
#   _ref/dym-mod-metro-gpu      the reference's dym-mod-metro with its two sweep
#                       loops turned into calls of oracle/ref_gpu_driver.cpp
#                       (dym_sweep_refarray on its own link array), streamed
#                       through sed into the compiler, linked with libdymgpu;
#                       built only when the engine's library has been built
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF_DIR=${REF_DIR:-$HERE/../baseline/_ref}
OUT="$HERE/_ref"
CORE="$HERE/../dym_symanzik_action_gb300/csrc"
CC=${CC:-gcc}
CXX=${CXX:-g++}
if [ ! -f "$REF_DIR/dym-mod-metro.cpp" ]; then
  echo "reference sources not found in $REF_DIR" >&2
  exit 2
fi
mkdir -p "$OUT"
# harness library (serial)
$CC -O2 -fPIC -std=gnu99 -w -c "$REF_DIR/group.c" -o "$OUT/h_group.o"
$CC -O2 -fPIC -std=gnu99 -w -c "$REF_DIR/lattice.c" -o "$OUT/h_lattice.o"
$CXX -O2 -fPIC -std=c++11 -w -ffp-contract=off -Dmain=dym_reference_main -I"$REF_DIR" \
  -c "$REF_DIR/dym-mod-metro.cpp" -o "$OUT/h_metro.o"
$CXX -O2 -fPIC -std=c++11 -w -c "$REF_DIR/timer.cpp" -o "$OUT/h_timer.o"
$CXX -O2 -fPIC -std=c++17 -ffp-contract=off -I"$REF_DIR" -I"$CORE" -c "$HERE/ref_harness.cpp" -o "$OUT/h_harness.o"
# -Bsymbolic: the reference's step() must not resolve to glibc's legacy
# regexp step() when the library is loaded into a running process.
$CXX -shared -Wl,-Bsymbolic -o "$OUT/libdymref.so" "$OUT/h_harness.o" "$OUT/h_metro.o" "$OUT/h_lattice.o" "$OUT/h_group.o" "$OUT/h_timer.o"
# unmodified executable, reference Makefile flags
$CC -O3 -std=gnu99 -Wall -fopenmp -w -c "$REF_DIR/group.c" -o "$OUT/group.o"
$CC -O3 -std=gnu99 -Wall -fopenmp -w -c "$REF_DIR/lattice.c" -o "$OUT/lattice.o"
$CXX -O3 -g -pg -fopenmp -std=c++11 -w -c "$REF_DIR/timer.cpp" -o "$OUT/timer.o"
$CXX -O3 -g -pg -fopenmp -std=c++11 -w -I"$REF_DIR" "$REF_DIR/dym-mod-metro.cpp" \
  "$OUT/lattice.o" "$OUT/group.o" "$OUT/timer.o" -lm -o "$OUT/dym-mod-metro"
sed 's/^#define NHIT[ \t]*20/#define NHIT 10/' "$REF_DIR/dym-mod-metro.cpp" | \
  $CXX -O3 -g -pg -fopenmp -std=c++11 -w -I"$REF_DIR" -x c++ - -x none \
  "$OUT/lattice.o" "$OUT/group.o" "$OUT/timer.o" -lm -o "$OUT/dym-mod-metro-nhit10"
$CXX -O3 -g -pg -fopenmp -std=c++11 -w -I"$REF_DIR" "$REF_DIR/llr.cpp" \
  "$OUT/lattice.o" "$OUT/group.o" "$OUT/timer.o" -lm -o "$OUT/llr"
$CXX -O3 -g -pg -fopenmp -std=c++11 -w -I"$REF_DIR" "$REF_DIR/llr2d.cpp" \
  "$OUT/lattice.o" "$OUT/group.o" "$OUT/timer.o" -lm -o "$OUT/llr2d"
# the reference's driver on the engine (needs lib/libdymgpu.so)
ENGINE_LIB="$CORE/../lib"
if [ -f "$ENGINE_LIB/libdymgpu.so" ]; then
  SRC="$REF_DIR/dym-mod-metro.cpp"
  THERM='for (unsigned k = 0; k < NTHERM; k++) update();'
  BLOCK='for (unsigned k = 0; k < K; k++) update();'
  if [ "$(grep -cF "$THERM" "$SRC")" != 1 ] || [ "$(grep -cF "$BLOCK" "$SRC")" != 1 ]; then
    echo "dym-mod-metro.cpp: sweep loops not found as expected; dym-mod-metro-gpu not built" >&2
    exit 3
  fi
  $CXX -O3 -std=c++17 -w -I"$REF_DIR" -I"$HERE/../include" -c "$HERE/ref_gpu_driver.cpp" -o "$OUT/ref_gpu_driver.o"
  sed -e '1i void dym_ref_sweeps(const char*, int, unsigned, int);' \
      -e 's/for (unsigned k = 0; k < NTHERM; k++) update();/dym_ref_sweeps(groupfilename, iseed, NTHERM, NHIT);/' \
      -e 's/for (unsigned k = 0; k < K; k++) update();/dym_ref_sweeps(groupfilename, iseed, K, NHIT);/' "$SRC" | \
    $CXX -O3 -fopenmp -std=c++11 -w -I"$REF_DIR" -x c++ - -x none "$OUT/ref_gpu_driver.o" \
      "$OUT/lattice.o" "$OUT/group.o" "$OUT/timer.o" -lm -L"$ENGINE_LIB" -ldymgpu -Wl,-rpath,"$ENGINE_LIB" \
      -o "$OUT/dym-mod-metro-gpu"
fi
echo "built $OUT"
