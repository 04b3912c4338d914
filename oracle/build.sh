#!/bin/sh
# Builds the CPU oracle (test infrastructure only) into oracle/_build/liboracle.so.
# The stroker source is the product's host-side input preparation, compiled in
# so that both renderers see identical stroke outlines.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
g++ -std=c++17 -O2 -fPIC -shared -ffp-contract=off -fno-fast-math -fwrapv -fno-strict-aliasing \
    -I"$HERE/../include" \
    "$HERE/raster.cpp" "$HERE/render.cpp" "$HERE/filter.cpp" "$HERE/soft.cpp" \
    "$HERE/../resvg_gb300/csrc/host/geom.cpp" "$HERE/../resvg_gb300/csrc/host/stroke.cpp" \
    "$HERE/../resvg_gb300/csrc/host/hairline.cpp" \
    "$HERE/../resvg_gb300/csrc/host/tree.cpp" \
    -o "$HERE/_build/liboracle.so.tmp" -lpthread
mv "$HERE/_build/liboracle.so.tmp" "$HERE/_build/liboracle.so"
