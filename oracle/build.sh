#!/bin/sh
# Builds the CPU oracle (test infrastructure only) into oracle/_build/liboracle.so.
# The stroker source is the product's host-side input preparation, compiled in
# so that both renderers see identical stroke outlines.  The synthetic scene
# generator (gen.cpp) is compiled in too, so the benchmark's reference arm
# builds the same trees without loading the product library.
# Translation units compile in parallel, then link.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
HOST="$HERE/../resvg_gb300/csrc/host"
OUT="$HERE/_build"
mkdir -p "$OUT/obj"
FLAGS="-std=c++17 -O2 -fPIC -ffp-contract=off -fno-fast-math -fwrapv -fno-strict-aliasing -I$HERE/../include"
SRCS="$HERE/raster.cpp $HERE/render.cpp $HERE/filter.cpp $HERE/soft.cpp $HERE/scenes.cpp \
      $HOST/geom.cpp $HOST/stroke.cpp $HOST/hairline.cpp $HOST/tree.cpp $HOST/gen.cpp"
PIDS=""
OBJS=""
for s in $SRCS; do
    o="$OUT/obj/$(basename "$s" .cpp).o"
    OBJS="$OBJS $o"
    g++ $FLAGS -c "$s" -o "$o" &
    PIDS="$PIDS $!"
done
FAIL=0
for p in $PIDS; do
    wait "$p" || FAIL=1
done
[ "$FAIL" = 0 ] || { echo "oracle: compile failed" >&2; exit 1; }
g++ -shared $OBJS -o "$OUT/liboracle.so.tmp" -lpthread
mv "$OUT/liboracle.so.tmp" "$OUT/liboracle.so"
