#!/usr/bin/env bash
# Builds the reference BatchLayout code from its own sources, where they lie,
# into oracle/_ref/ (git-ignored).  Never writes into the reference tree and
# never runs the reference's own build system.  Test infrastructure only.
#
#   oracle/_ref/BatchLayout         stock flags of the reference Makefile
#                                   (-O3 -ffast-math -fopenmp -DCPP, plus
#                                   -mavx512f -mavx512dq on x86_64 only)
#   oracle/_ref/BatchLayout_strict  same sources, no fast-math, no FMA contraction
#   oracle/_ref/ref_driver          oracle/ref_driver.cpp + sample/algorithms.cpp,
#                                   strict flags: full-precision golden vectors
#
# usage: oracle/build_ref.sh REFERENCE_DIR   (or BL_REFERENCE_DIR in the environment)
set -euo pipefail
REF="${1:-${BL_REFERENCE_DIR:-}}"
if [ -z "$REF" ]; then
  echo "usage: $0 REFERENCE_DIR (or set BL_REFERENCE_DIR)" >&2
  exit 2
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/sample/algorithms.cpp" ]; then
  echo "reference sources not found at $REF; nothing to build" >&2
  exit 3
fi
mkdir -p "$OUT"
INC="-I$REF -I$REF/sample -I$REF/Test"
ARCHF=""
if [ "$(uname -m)" = "x86_64" ]; then ARCHF="-mavx512f -mavx512dq"; fi
STOCK="-g -fomit-frame-pointer -fopenmp -ffast-math $ARCHF -O3 -std=c++11 -DCPP -w"
STRICT="-O2 -fopenmp -std=c++11 -DCPP -ffp-contract=off -w"
g++ $INC $STOCK  -o "$OUT/BatchLayout"        "$REF/sample/algorithms.cpp" "$REF/Test/BatchLayout.cpp" &
g++ $INC $STRICT -o "$OUT/BatchLayout_strict" "$REF/sample/algorithms.cpp" "$REF/Test/BatchLayout.cpp" &
g++ $INC $STRICT -o "$OUT/ref_driver"         "$HERE/ref_driver.cpp" "$REF/sample/algorithms.cpp" &
wait
echo "built: $(ls "$OUT")"
