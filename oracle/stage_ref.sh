#!/bin/sh
# Places the unmodified reference files that the checkers and the reference
# arm of bench.py need into baseline/_ref/ (git-ignored, never committed; it
# travels with the working tree to the GPU machine, where oracle/build_ref.sh
# compiles them for that machine).  The reference is a C/C++ tree without
# Python packaging, so `pip install --target baseline/_ref` cannot install it;
# this script is the install step instead.  Nothing is edited: the files are
# copied byte for byte and their SHA-256 sums recorded in baseline/_ref/SHA256SUMS.
#
#   sh oracle/stage_ref.sh <reference checkout>
set -e
SRC=${1:-$REF_SRC}
if [ -z "$SRC" ] || [ ! -f "$SRC/dym-mod-metro.cpp" ]; then
  echo "usage: sh oracle/stage_ref.sh <reference checkout>  (dym-mod-metro.cpp not found)" >&2
  exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
DST="$HERE/../baseline/_ref"
mkdir -p "$DST/groups" "$DST/scripts"
# sources of the path (Makefile flags are read from the Makefile itself)
for f in Makefile group.c group.h lattice.c lattice.h timer.cpp timer.h dym-mod-metro.cpp llr.cpp llr2d.cpp \
         verify_group.c; do
  cp "$SRC/$f" "$DST/$f"
done
# the table files the tests and benchmarks load
for f in mys1080-v4 myBI myBT myBO S648 S108 siii_360x4 svii_120x4 sviii_120x4 si_60x4; do
  cp "$SRC/groups/$f" "$DST/groups/$f"
done
# the log consumers whose parsing must keep working on the engine's output
for f in getavgsimpplaq.py pltabsvalpolyakov.py llr_reconstruct.py; do
  cp "$SRC/scripts/$f" "$DST/scripts/$f"
done
chmod -R u+w "$DST"
(cd "$DST" && find . -type f ! -name SHA256SUMS | sort | xargs sha256sum > SHA256SUMS)
echo "staged $(wc -l < "$DST/SHA256SUMS") reference files into $DST"
