#!/bin/sh
# ORACLE — test infrastructure.  Compiles the reference's gradient.cpp (unmodified, read where it
# lies) into oracle/_ref/libvvref_sobel.so and oracle/_ref/libvvref_central.so.
#
# The reference is a Windows GL application; gradient.cpp itself calls no GL function, but its
# headers include GL headers by Windows-style names.  The include shim generated below only maps
# those names (`GL\glew.h` with a backslash, `dataSet.h` vs dataset.h) onto the GLEW header the
# reference vendors and an empty freeglut header.  Nothing here provides or loads any graphics
# library.  Usage: sh oracle/build_ref.sh <reference-root>   (or $VVLIC_REFERENCE_ROOT)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=${1:-$VVLIC_REFERENCE_ROOT}
if [ -z "$ROOT" ]; then
  echo "build_ref: give the reference checkout as the argument or in VVLIC_REFERENCE_ROOT" >&2
  exit 2
fi
SRC="$ROOT/VectorVisualization"
OUT="$HERE/_ref"
if [ ! -f "$SRC/gradient.cpp" ]; then
  echo "build_ref: reference sources not found under $ROOT" >&2
  exit 2
fi
mkdir -p "$OUT/shim/GL"
printf '#include <GL/glew.h>\n' > "$OUT/shim/GL\\glew.h"
: > "$OUT/shim/GL\\freeglut.h"
: > "$OUT/shim/GL/freeglut.h"
printf '#include "dataset.h"\n' > "$OUT/shim/dataSet.h"
CXX=${CXX:-g++}
FLAGS="-O2 -std=c++14 -fPIC -shared -ffp-contract=off -w -DGLEW_NO_GLU -DGLEW_STATIC"
INC="-I$OUT/shim -I$SRC -I$SRC/glew-1.11.0/include"
$CXX $FLAGS $INC "$HERE/ref_driver.cpp" "$SRC/reader.cpp" -o "$OUT/libvvref_sobel.so"
$CXX $FLAGS $INC -DVVREF_CENTRAL "$HERE/ref_driver.cpp" "$SRC/reader.cpp" -o "$OUT/libvvref_central.so"
echo "build_ref: built $OUT/libvvref_sobel.so $OUT/libvvref_central.so"
